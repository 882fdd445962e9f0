"""Golden vectors for the hash-grid texture from the reference's own
``MLPTexture3D`` (geo/texture.py), run on the CPU.

    python tests/golden/make_texture_golden.py [/path/to/reference]

tiny-cuda-nn is not installed, so a stand-in ``tinycudann`` module provides
``Encoding`` computed by the oracle's restatement of the hash-grid encoding
(``oracle/texture.py``).  What this pins is the reference code around the
encoding: the AABB normalisation and clamp, the MLP (``_MLP``), the output
layout of ``sample_noact`` and the two gradient-scaling hooks.  The
encoding's table is a closed-form pattern (``pattern_table``) so the
fixture need not store its 6.3M entries.  Output: ``texture_golden.npz``:
inputs (points, AABB, MLP weights), features, upstream gradient, and
gradients w.r.t. the points, the MLP weights and the table (as nonzero
entries).
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import texture as otex  # noqa: E402
from tests.golden.make_golden import CpuRedirect  # noqa: E402


def pattern_table(entries):
    """Deterministic table values: 0.1 sin(12.9898 i + 78.233 f)."""
    i = np.arange(entries, dtype=np.float64)[:, None]
    f = np.arange(2, dtype=np.float64)[None, :]
    return (0.1 * np.sin(12.9898 * i + 78.233 * f)).astype(np.float32)


class StandInEncoding(torch.nn.Module):
    """tinycudann.Encoding stand-in: the oracle's hash-grid encoding."""

    def __init__(self, n_input_dims, encoding_config, seed=1337, dtype=None):
        super().__init__()
        assert n_input_dims == 3 and encoding_config["otype"] == "HashGrid"
        assert encoding_config["n_levels"] == otex.N_LEVELS
        assert encoding_config["n_features_per_level"] == otex.N_FEATURES
        assert encoding_config["log2_hashmap_size"] == otex.LOG2_HASHMAP
        assert encoding_config["base_resolution"] == otex.BASE_RES
        assert abs(encoding_config["per_level_scale"] - otex.per_level_scale()) < 1e-12
        n = otex.table_entries()
        self.params = torch.nn.Parameter(torch.tensor(pattern_table(n)).reshape(-1))
        self.n_output_dims = otex.N_LEVELS * otex.N_FEATURES

    def forward(self, x):
        return otex.encode(x, self.params.view(-1, 2))


def main(ref):
    sys.modules["tinycudann"] = types.SimpleNamespace(Encoding=StandInEncoding,
                                                      free_temporary_memory=lambda: None)
    sys.path.insert(0, ref)
    with CpuRedirect():
        from geo.texture import MLPTexture3D
        torch.manual_seed(0)
        aabb = torch.tensor([[-1.0, -0.9, -1.1], [1.05, 1.0, 0.95]]) * 1.1
        tex = MLPTexture3D(aabb, channels=48, min_max=None)
        rng = np.random.default_rng(5)
        xyz = torch.tensor(rng.uniform(-1.3, 1.3, (96, 3)).astype(np.float32), requires_grad=True)
        out = tex.sample_noact(xyz)
        up = torch.tensor(rng.standard_normal(tuple(out.shape)).astype(np.float32))
        (out * up).sum().backward()
    W = [tex.net.net[k].weight for k in (0, 2, 4)]
    dt = tex.encoder.params.grad.view(-1, 2)
    nz = torch.nonzero(dt.abs().sum(1) > 0).squeeze(1)
    np.savez_compressed(
        os.path.join(HERE, "texture_golden.npz"),
        aabb=aabb.numpy(), xyz=xyz.detach().numpy(), W1=W[0].detach().numpy(),
        W2=W[1].detach().numpy(), W3=W[2].detach().numpy(), out=out.detach().numpy(),
        up=up.numpy(), dxyz=xyz.grad.numpy(), dW1=W[0].grad.numpy(), dW2=W[1].grad.numpy(),
        dW3=W[2].grad.numpy(), dtable_idx=nz.numpy().astype(np.int64),
        dtable_val=dt[nz].numpy(), state_keys=np.array(sorted(tex.state_dict().keys())))
    print("features", tuple(out.shape), "table entries touched", int(nz.numel()))


if __name__ == "__main__":
    ref_tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMGS_REFERENCE_TREE")
    if not ref_tree:
        sys.exit(f"usage: python {os.path.basename(__file__)} <reference tree> "
                 "(or set DMGS_REFERENCE_TREE)")
    main(ref_tree)
