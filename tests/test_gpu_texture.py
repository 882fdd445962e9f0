"""Hash-grid texture kernels (csrc/texture.cu through the C ABI) against the
reference wrapper's golden vectors and the oracle run in float32.

Tolerances: features within 2e-6 absolute of the float32 references (the
encoding's operations are mirrored; the MLP sums in another order);
gradients within 1e-4 relative L2 (float atomics)."""
import os

import numpy as np
import pytest
import torch

from oracle import texture as otex
from tests.golden.make_texture_golden import pattern_table

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "texture_golden.npz")


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def make_texture(aabb, channels, W=None, table=None):
    from dmgs_gb300.texture import MLPTexture3D
    tex = MLPTexture3D(torch.tensor(aabb), channels=channels)
    with torch.no_grad():
        if table is not None:
            tex.encoder.params.copy_(torch.tensor(table).reshape(-1))
        if W is not None:
            for w, v in zip(tex.net.weights(), W):
                w.copy_(torch.tensor(v))
    return tex


def test_matches_reference_wrapper():
    z = np.load(GOLDEN)
    table = pattern_table(otex.table_entries())
    tex = make_texture(z["aabb"], 48, [z["W1"], z["W2"], z["W3"]], table)
    xyz = torch.tensor(z["xyz"], device="cuda", requires_grad=True)
    out = tex.sample_noact(xyz)
    assert np.abs(out.detach().cpu().numpy() - z["out"]).max() <= 2e-6
    (out * torch.tensor(z["up"], device="cuda")).sum().backward()
    assert rel_l2(xyz.grad.cpu(), z["dxyz"]) < 1e-4
    for k, w in zip(("dW1", "dW2", "dW3"), tex.net.weights()):
        assert rel_l2(w.grad.cpu(), z[k]) < 1e-4, k
    dt = tex.encoder.params.grad.view(-1, 2).cpu()
    nz = torch.nonzero(dt.abs().sum(1) > 0).squeeze(1).numpy()
    assert np.array_equal(nz, z["dtable_idx"])
    assert rel_l2(dt[nz], z["dtable_val"]) < 1e-4


@pytest.mark.parametrize("channels,n", [(48, 65536), (27, 3000), (12, 1000), (3, 777)])
def test_matches_oracle(channels, n):
    rng = np.random.default_rng(channels)
    aabb = np.array([[-1.2, -1.1, -1.0], [1.1, 1.2, 1.3]], np.float32)
    table = rng.normal(0, 0.05, (otex.table_entries(), 2)).astype(np.float32)
    W = [rng.normal(0, 0.3, s).astype(np.float32) for s in ((32, 32), (32, 32), (channels, 32))]
    xyz = rng.uniform(-1.3, 1.4, (n, 3)).astype(np.float32)  # some outside the box
    up = rng.standard_normal((n, channels)).astype(np.float32)
    tex = make_texture(aabb, channels, W, table)
    x = torch.tensor(xyz, device="cuda", requires_grad=True)
    out = tex.sample_noact(x)
    (out * torch.tensor(up, device="cuda")).sum().backward()
    t = lambda a: torch.tensor(a, dtype=torch.float32, requires_grad=True)
    xo, to, Wo = t(xyz), t(table), [t(w) for w in W]
    oo = otex.sample_noact(xo, torch.tensor(aabb), to, Wo)
    (oo * torch.tensor(up)).sum().backward()
    assert np.abs(out.detach().cpu().numpy() - oo.detach().numpy()).max() <= 2e-6
    assert rel_l2(x.grad.cpu(), xo.grad) < 1e-4
    for w, wo in zip(tex.net.weights(), Wo):
        assert rel_l2(w.grad.cpu(), wo.grad) < 1e-4
    assert rel_l2(tex.encoder.params.grad.view(-1, 2).cpu(), to.grad) < 1e-4


def test_state_dict_and_empty_input():
    tex = make_texture(np.array([[-1, -1, -1], [1, 1, 1]], np.float32), 48)
    assert sorted(tex.state_dict().keys()) == ["encoder.params", "net.net.0.weight",
                                               "net.net.2.weight", "net.net.4.weight"]
    assert tex.encoder.params.numel() == 2 * otex.table_entries()
    out = tex.sample_noact(torch.zeros((0, 3), device="cuda"))
    assert out.shape == (0, 48)


def test_kept_encoding_gives_the_recomputed_gradients():
    """dmgs_tex_fwd_enc + dmgs_tex_bwd_enc (the encoding kept from the
    forward) against dmgs_tex_fwd + dmgs_tex_bwd (recomputed in the adjoint)
    through the C ABI: the same outputs, the same per-point encoding
    gradients and position gradients bit for bit, the weight and table
    gradients equal up to the order of their float atomics."""
    import ctypes as C
    from dmgs_gb300 import _lib
    from dmgs_gb300._lib import check, ptr, stream_of
    from dmgs_gb300.texture import _desc
    lib = _lib.load()
    rng = np.random.default_rng(7)
    n, channels = 20000, 48
    aabb = torch.tensor([[-1.0, -1.0, -1.0], [1.0, 1.0, 1.0]])
    table = torch.tensor(rng.normal(0, 0.05, (otex.table_entries(), 2)).astype(np.float32), device="cuda")
    W = [torch.tensor(rng.normal(0, 0.3, s).astype(np.float32), device="cuda")
         for s in ((32, 32), (32, 32), (channels, 32))]
    xyz = torch.tensor(rng.uniform(-1.1, 1.1, (n, 3)).astype(np.float32), device="cuda")
    up = torch.tensor(rng.standard_normal((n, channels)).astype(np.float32), device="cuda")
    pls = float(np.exp(np.log(4096 / 16) / 15))
    d = _desc(aabb, table, *W, channels, pls)
    s = stream_of(xyz.device)
    res = []
    for keep in (False, True):
        out = torch.empty((n, channels), device="cuda")
        enc = torch.empty((n, 32), device="cuda") if keep else None
        if keep:
            check(lib.dmgs_tex_fwd_enc(C.byref(d), n, ptr(xyz), ptr(out), ptr(enc), s), "fwd")
        else:
            check(lib.dmgs_tex_fwd(C.byref(d), n, ptr(xyz), ptr(out), s), "fwd")
        dx, dt = torch.empty_like(xyz), torch.empty_like(table)
        dw = [torch.empty_like(w) for w in W]
        scratch = torch.empty(lib.dmgs_tex_bwd_scratch_bytes(n) // 4, device="cuda")
        args = (ptr(up), ptr(dx), ptr(dt), *(w.data_ptr() for w in dw), scratch.data_ptr(),
                scratch.numel() * 4, s)
        if keep:
            check(lib.dmgs_tex_bwd_enc(C.byref(d), n, ptr(xyz), ptr(enc), *args), "bwd")
        else:
            check(lib.dmgs_tex_bwd(C.byref(d), n, ptr(xyz), *args), "bwd")
        torch.cuda.synchronize()
        res.append((out, scratch, dx, dt, dw))
    (o0, e0, x0, t0, w0), (o1, e1, x1, t1, w1) = res
    assert torch.equal(o0, o1)
    assert torch.equal(e0, e1)  # dL/denc per point
    assert torch.equal(x0, x1)
    assert rel_l2(t1.cpu(), t0.cpu()) < 1e-6
    for a, b in zip(w1, w0):
        assert rel_l2(a.cpu(), b.cpu()) < 1e-6
