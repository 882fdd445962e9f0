"""Hash-grid texture oracle against the reference's own MLPTexture3D (CPU).

The golden file comes from the reference's ``geo/texture.py`` run with the
oracle's encoding standing in for tiny-cuda-nn, so this pins the code around
the encoding (normalisation, clamp, MLP, hooks, layout); the encoding itself
is a restatement of the published algorithm (parity unpinned)."""
import os

import numpy as np
import torch

from oracle import texture as otex
from tests.golden.make_texture_golden import pattern_table

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "texture_golden.npz")


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_layout():
    lay = otex.level_layout()
    res = [r for _, r, _, _, _ in lay]
    assert res[0] == 16 and res[-1] in (4096, 4097)
    assert [h for *_, h in lay] == [False] * 5 + [True] * 11
    assert all(size % 8 == 0 for _, _, _, size, _ in lay)
    assert otex.table_entries() == sum(size for _, _, _, size, _ in lay)


def run(z, dtype):
    t = lambda k: torch.tensor(z[k], dtype=dtype, requires_grad=True)
    xyz, W = t("xyz"), [t("W1"), t("W2"), t("W3")]
    table = torch.tensor(pattern_table(otex.table_entries()), dtype=dtype, requires_grad=True)
    out = otex.sample_noact(xyz, torch.tensor(z["aabb"], dtype=dtype), table, W)
    (out * torch.tensor(z["up"], dtype=dtype)).sum().backward()
    return out.detach(), xyz, W, table


def test_float64_oracle_near_reference_wrapper():
    """Float32 positions carry ~2.4e-4 cell fractions at the finest level
    (scale 4095), which bounds any float32 run's agreement with float64."""
    z = np.load(GOLDEN)
    out, xyz, W, table = run(z, torch.float64)
    assert np.abs(out.numpy() - z["out"]).max() < 2e-4
    assert rel_l2(xyz.grad, z["dxyz"]) < 1e-2


def test_sample_noact_matches_reference_wrapper():
    z = np.load(GOLDEN)
    out, xyz, W, table = run(z, torch.float32)
    assert np.abs(out.numpy() - z["out"]).max() < 1e-6
    assert rel_l2(xyz.grad, z["dxyz"]) < 1e-4
    for k, w in zip(("dW1", "dW2", "dW3"), W):
        assert rel_l2(w.grad, z[k]) < 1e-4, k
    dt = table.grad
    nz = torch.nonzero(dt.abs().sum(1) > 0).squeeze(1).numpy()
    assert np.array_equal(nz, z["dtable_idx"])
    assert rel_l2(dt[nz], z["dtable_val"]) < 1e-4


def test_state_dict_keys():
    z = np.load(GOLDEN)
    assert list(z["state_keys"]) == ["encoder.params", "net.net.0.weight", "net.net.2.weight",
                                     "net.net.4.weight"]
