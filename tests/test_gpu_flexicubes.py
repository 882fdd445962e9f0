"""FlexiCubes CUDA path (csrc/flexicubes.cu through the C ABI) against the
reference's own outputs (golden file) and the float64 oracle.

Tolerances: integer outputs (faces, surface edges) exact; vertices and L_dev
within 2e-6 absolute of the reference (float32 both) and 2e-5 of the float64
oracle; gradients within 1e-4 relative L2 (float atomics change the
summation order) of the reference and of the oracle run in float32, the
reference's precision.  Against a float64 run the gradients can differ by
more: L_dev = |dist - mean| is not differentiable where a distance equals
its mean, and such near-ties are resolved by float32 rounding the same way
here as in a float32 run of the reference algorithm.
"""
import os

import numpy as np
import pytest
import torch

from oracle import flexicubes as ofc

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "flexicubes_golden.npz")


def fc():
    from dmgs_gb300.flexicubes import flexicubes
    return flexicubes


def load(case):
    z = np.load(GOLDEN)
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(case + "/")}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def run_gpu(d, grad=False):
    dev = "cuda"
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=grad)
    x, s = t(d["x"]), t(d["s"])
    w = [t(d[k]) if d.get(k) is not None else None for k in ("beta", "alpha", "gamma")]
    out = fc()(x, s, tuple(int(r) for r in d["res"]), *w, training=bool(d["training"]))
    return out, [x, s] + w


def run_oracle(d, grad=False, dtype=torch.float64):
    t = lambda a: torch.tensor(np.asarray(a), dtype=dtype, requires_grad=grad)
    x, s = t(d["x"]), t(d["s"])
    w = [t(d[k]) if d.get(k) is not None else None for k in ("beta", "alpha", "gamma")]
    res = tuple(int(r) for r in d["res"])
    _, cubes = ofc.voxel_grid(res)
    out = ofc.extract(x, s, cubes, res, *w, training=bool(d["training"]))
    return out, [x, s] + w


def grads_of(out, inputs, up_v, up_L):
    v, f, L, se = out
    loss = (v * up_v.to(v)).sum() + (L * up_L.to(L)).sum()
    used = [i for i in inputs if i is not None]
    g = torch.autograd.grad(loss, used, allow_unused=True)
    it = iter(g)
    return [next(it) if i is not None else None for i in inputs]


@pytest.mark.parametrize("case", ("shape", "noise", "plain"))
def test_forward_matches_reference(case):
    d = load(case)
    (v, f, L, se), _ = run_gpu(d)
    torch.cuda.synchronize()
    assert np.array_equal(se.cpu().numpy(), d["surf_edges"])
    assert np.array_equal(f.cpu().numpy(), d["faces"])
    assert v.shape == d["vertices"].shape
    assert np.abs(v.cpu().numpy() - d["vertices"]).max() <= 2e-6
    assert np.abs(L.cpu().numpy() - d["L_dev"]).max() <= 2e-6
    if case == "plain":  # weights of exactly one: the same float32 operations as the reference
        assert np.array_equal(v.cpu().numpy(), d["vertices"])


@pytest.mark.parametrize("case", ("shape", "noise"))
def test_gradients_match_reference(case):
    d = load(case)
    out, inputs = run_gpu(d, grad=True)
    g = grads_of(out, inputs, torch.tensor(d["up_vertices"]), torch.tensor(d["up_L_dev"]))
    for name, gi in zip(("dx", "ds", "dbeta", "dalpha", "dgamma"), g):
        assert rel_l2(gi.cpu().numpy(), d[name]) < 1e-4, name


def synthetic(res, field, weights, training, seed):
    """Seeded grid inputs.  The shape field is offset by 3.7e-4 so that no
    grid vertex sits on the surface: where |s| ~ 1e-8 (an axis vertex of the
    sphere) the float32 adjoint w.r.t. s is ill-conditioned for the
    reference's float32 arithmetic as much as for this one."""
    rng = np.random.default_rng(seed)
    verts, _ = ofc.voxel_grid(res, (-1, -1, -1), (1, 1, 1))
    p = verts.numpy().astype(np.float64)
    if field == "shape":
        sph = np.linalg.norm(p, axis=1) - 0.6
        q = np.stack([np.hypot(p[:, 0], p[:, 1]) - 0.7, p[:, 2]], 1)
        s = np.minimum(sph, np.linalg.norm(q, axis=1) - 0.2) + 3.7e-4
        assert np.abs(s).min() > 1e-6
    else:
        s = rng.standard_normal(p.shape[0])
    cube = 2.0 / max(res)
    x = p + rng.uniform(-0.2, 0.2, p.shape) * cube
    C = res[0] * res[1] * res[2]
    d = {"res": np.array(res), "x": x.astype(np.float32), "s": s.astype(np.float32),
         "training": np.array(training)}
    if weights:
        d.update(beta=rng.normal(0, 0.7, (C, 12)).astype(np.float32),
                 alpha=rng.normal(0, 0.7, (C, 8)).astype(np.float32),
                 gamma=rng.normal(0, 0.7, (C,)).astype(np.float32))
    return d


@pytest.mark.parametrize("res,field,weights,training", [
    ((24, 31, 27), "noise", True, True),
    ((40, 36, 44), "shape", True, True),
    ((33, 20, 25), "noise", True, False),
    ((64, 64, 64), "shape", False, True),
])
def test_matches_oracle(res, field, weights, training):
    d = synthetic(res, field, weights, training, seed=sum(res))
    (v, f, L, se), gin = run_gpu(d, grad=True)
    (vo, fo, Lo, seo), _ = run_oracle(d)
    assert np.array_equal(se.detach().cpu().numpy(), seo.numpy())
    assert np.array_equal(f.cpu().numpy(), fo.numpy())
    assert np.abs(v.detach().cpu().double().numpy() - vo.detach().numpy()).max() <= 2e-5
    assert np.abs(L.detach().cpu().double().numpy() - Lo.detach().numpy()).max() <= 2e-5
    if not training:
        return
    rng = np.random.default_rng(7)
    up_v = torch.tensor(rng.standard_normal(tuple(v.shape)))
    up_L = torch.tensor(rng.standard_normal(tuple(L.shape)))
    g = grads_of((v, f, L, se), gin, up_v, up_L)
    out32, oin = run_oracle(d, grad=True, dtype=torch.float32)
    go = grads_of(out32, oin, up_v, up_L)
    for name, a, b in zip(("dx", "ds", "dbeta", "dalpha", "dgamma"), g, go):
        if b is None:
            continue
        assert rel_l2(a.cpu().numpy(), b.numpy()) < 1e-4, name


def test_configuration_mesh_size():
    """Sphere(0.6) union torus(0.7, 0.2) on a 64^3 grid over [-1,1]^3 in
    training mode: ~45k triangles, a closed manifold (each edge in two faces)."""
    d = synthetic((64, 64, 64), "shape", False, True, seed=0)
    d["x"] = ofc.voxel_grid((64, 64, 64), (-1, -1, -1), (1, 1, 1))[0].numpy()
    (v, f, L, se), _ = run_gpu(d)
    F = f.shape[0]
    assert 40000 < F < 50000
    e = torch.cat([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]).sort(1).values
    _, cnt = torch.unique(e, dim=0, return_counts=True)
    assert bool((cnt == 2).all())


def test_no_surface():
    d = synthetic((5, 6, 7), "noise", True, True, seed=3)
    d["s"] = np.abs(d["s"]) + 0.1
    (v, f, L, se), _ = run_gpu(d)
    assert v.shape == (0, 3) and f.shape == (0, 3) and L.shape == (0,) and se is None


def test_class_interface():
    from dmgs_gb300.flexicubes import FlexiCubes
    m = FlexiCubes()
    verts, cubes = m.construct_voxel_grid_v2([6, 5, 4], [-1, -1, -1], [1, 1, 1])
    ov, oc = ofc.voxel_grid((6, 5, 4), (-1, -1, -1), (1, 1, 1))
    assert torch.equal(cubes.cpu().long(), oc)
    assert torch.allclose(verts.cpu(), ov, atol=1e-6)
    s = verts.norm(dim=1) - 0.7
    v, f, L, se = m(verts, s, cubes, [6, 5, 4], training=True)
    assert f.shape[0] > 0 and se.shape[1] == 2
    with pytest.raises(NotImplementedError):
        m(verts, s, cubes.flip(0), [6, 5, 4])
    with pytest.raises(NotImplementedError):
        m(verts, s, cubes, [6, 5, 4], output_tetmesh=True)


def test_weight_slices_of_one_tensor_read_in_place():
    """Stage 2 passes per_cube_weights[:, :12], [:, 12:20], [:, 20] (one
    [C, 21] tensor): the kernels then read and write it in place.  Same
    outputs and gradients as separate dense weight tensors."""
    res = (20, 24, 22)
    d = synthetic(res, "shape", True, True, seed=9)
    dev = "cuda"
    x = torch.tensor(d["x"], device=dev, requires_grad=True)
    s = torch.tensor(d["s"], device=dev, requires_grad=True)
    Wd = torch.cat([torch.tensor(d["beta"]), torch.tensor(d["alpha"]),
                    torch.tensor(d["gamma"])[:, None]], 1).to(dev)
    W = Wd.clone().requires_grad_(True)
    sep = [Wd[:, :12].clone().requires_grad_(True), Wd[:, 12:20].clone().requires_grad_(True),
           Wd[:, 20].clone().requires_grad_(True)]
    out_w = fc()(x, s, res, W[:, :12], W[:, 12:20], W[:, 20], training=True)
    out_s = fc()(x.detach().requires_grad_(True), s.detach().requires_grad_(True), res, *sep,
                 training=True)
    for a, b in zip(out_w, out_s):
        assert torch.equal(a, b)
    rng = np.random.default_rng(1)
    up_v = torch.tensor(rng.standard_normal(tuple(out_w[0].shape)), dtype=torch.float32, device=dev)
    up_L = torch.tensor(rng.standard_normal(tuple(out_w[2].shape)), dtype=torch.float32, device=dev)
    ((out_w[0] * up_v).sum() + (out_w[2] * up_L).sum()).backward()
    ((out_s[0] * up_v).sum() + (out_s[2] * up_L).sum()).backward()
    ref = torch.cat([sep[0].grad, sep[1].grad, sep[2].grad[:, None]], 1)
    assert rel_l2(W.grad.cpu().numpy(), ref.cpu().numpy()) < 1e-6
