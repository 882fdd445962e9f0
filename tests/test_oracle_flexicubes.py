"""FlexiCubes oracle pinned to the reference (CPU only).

The golden file holds the reference class's own outputs and autograd
gradients (``tests/golden/make_flexicubes_golden.py``).  Integer outputs
(faces, surface edges) must match exactly; float outputs to float32
rounding (the oracle runs in float64, the reference in float32).
"""
import os

import numpy as np
import pytest
import torch

from oracle import flexicubes as ofc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "flexicubes_golden.npz")
# the reference tree (read-only), located through the environment; the tests
# that run the reference's own code skip without it
REF_ROOT = os.environ.get("DMGS_REFERENCE_TREE", "")
REF_TABLES = os.path.join(REF_ROOT, "geo", "tables.py") if REF_ROOT else ""
CASES = ("shape", "noise", "plain")


def load(case):
    z = np.load(GOLDEN)
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(case + "/")}


def run_oracle(d, dtype=torch.float64, grad=False):
    t = lambda a: torch.tensor(a, dtype=dtype, requires_grad=grad)
    x, s = t(d["x"]), t(d["s"])
    w = [t(d[k]) if k in d else None for k in ("beta", "alpha", "gamma")]
    out = ofc.extract(x, s, torch.tensor(d["cubes"]), tuple(int(r) for r in d["res"]), *w,
                      training=bool(d["training"]))
    return out, [x, s] + w


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_tables_match_reference():
    if not REF_TABLES or not os.path.exists(REF_TABLES):
        pytest.skip("reference tree not present (set DMGS_REFERENCE_TREE)")
    ns = {}
    exec(compile(open(REF_TABLES).read(), REF_TABLES, "exec"), ns)
    dmc, num_vd, check = ofc.derive_tables()
    assert dmc == ns["dmc_table"]
    assert num_vd == ns["num_vd_table"]
    assert check == ns["check_table"]


def test_voxel_grid_matches_golden_cubes():
    d = load("shape")
    verts, cubes = ofc.voxel_grid(tuple(int(r) for r in d["res"]), (-1, -1, -1), (1, 1, 1))
    assert np.array_equal(cubes.numpy(), d["cubes"])


@pytest.mark.parametrize("case", CASES)
def test_forward_matches_reference(case):
    d = load(case)
    (v, f, L, se), _ = run_oracle(d)
    assert np.array_equal(se.numpy(), d["surf_edges"])
    assert np.array_equal(f.numpy(), d["faces"])
    assert v.shape == d["vertices"].shape
    assert np.abs(v.numpy() - d["vertices"]).max() < 2e-6
    assert np.abs(L.numpy() - d["L_dev"]).max() < 2e-6


@pytest.mark.parametrize("case", ("shape", "noise"))
def test_gradients_match_reference(case):
    d = load(case)
    (v, f, L, se), inputs = run_oracle(d, grad=True)
    loss = (v * torch.tensor(d["up_vertices"], dtype=v.dtype)).sum() + \
        (L * torch.tensor(d["up_L_dev"], dtype=L.dtype)).sum()
    grads = torch.autograd.grad(loss, inputs)
    for name, g in zip(("dx", "ds", "dbeta", "dalpha", "dgamma"), grads):
        assert rel_l2(g.numpy(), d[name]) < 1e-4, name


def test_no_surface_is_empty():
    verts, cubes = ofc.voxel_grid((3, 3, 3))
    s = torch.ones(verts.shape[0], dtype=torch.float64)
    v, f, L, se = ofc.extract(verts.double(), s, cubes, (3, 3, 3))
    assert v.shape == (0, 3) and f.shape == (0, 3) and L.shape == (0,) and se.shape == (0, 2)


@pytest.mark.parametrize("res,training", [((64, 64, 64), True), ((40, 36, 44), False),
                                          ((33, 48, 27), True)])
def test_oracle_matches_reference_class(res, training):
    """The oracle against the reference's own FlexiCubes class run here (when
    the reference tree is present): the configuration-2 grid (64^3 over
    [-1,1]^3, training mode) and two non-cubic grids (one in each
    quad-splitting mode), the sphere-union-torus field, deformed vertices and
    random weights; both in float32."""
    import sys
    ref_root = REF_ROOT
    if not ref_root or not os.path.exists(os.path.join(ref_root, "geo", "flexicubes.py")):
        pytest.skip("reference tree not present (set DMGS_REFERENCE_TREE)")
    sys.path.insert(0, ref_root)
    try:
        from geo.flexicubes import FlexiCubes
    finally:
        sys.path.remove(ref_root)
    rfc = FlexiCubes(device="cpu")
    verts, cubes = rfc.construct_voxel_grid_v2(list(res), [-1.0] * 3, [1.0] * 3)
    rng = np.random.default_rng(sum(res))
    p = verts.numpy().astype(np.float64)
    sph = np.linalg.norm(p, axis=1) - 0.6
    q = np.stack([np.hypot(p[:, 0], p[:, 1]) - 0.7, p[:, 2]], 1)
    s_np = (np.minimum(sph, np.linalg.norm(q, axis=1) - 0.2) + 3.7e-4).astype(np.float32)
    x_np = (p + rng.uniform(-0.2, 0.2, p.shape) * (2.0 / max(res))).astype(np.float32)
    C = cubes.shape[0]
    w_np = [rng.normal(0, 0.7, shp).astype(np.float32) for shp in ((C, 12), (C, 8), (C,))]

    def run(fn, cubes_t):
        t = lambda a: torch.tensor(a, requires_grad=True)  # noqa: E731
        x, s = t(x_np), t(s_np)
        w = [t(a) for a in w_np]
        out = fn(x, s, cubes_t, res, *w)
        up = np.random.default_rng(7)
        loss = (out[0] * torch.tensor(up.standard_normal(tuple(out[0].shape)), dtype=torch.float32)).sum() \
            + (out[2] * torch.tensor(up.standard_normal(tuple(out[2].shape)), dtype=torch.float32)).sum()
        # without training the split weights gamma only choose a diagonal: no gradient
        gs = torch.autograd.grad(loss, [x, s] + w, allow_unused=True)
        return out, [torch.zeros_like(t) if g is None else g for g, t in zip(gs, [x, s] + w)]

    (rv, rf, rL, rse), rg = run(lambda x, s, c, r, b, a, g: rfc(x, s, c, list(r), b, a, g,
                                                                training=training), cubes)
    (ov, of, oL, ose), og = run(lambda x, s, c, r, b, a, g: ofc.extract(x, s, c, r, b, a, g,
                                                                        training=training),
                                ofc.voxel_grid(res, (-1, -1, -1), (1, 1, 1))[1])
    assert np.array_equal(rse.numpy(), ose.numpy())
    assert np.array_equal(rf.numpy(), of.numpy())
    assert np.abs(rv.detach().numpy() - ov.detach().numpy()).max() < 2e-6
    assert np.abs(rL.detach().numpy() - oL.detach().numpy()).max() < 2e-6
    for name, a, b in zip(("dx", "ds", "dbeta", "dalpha", "dgamma"), og, rg):
        if not b.any():
            assert not a.any(), name
            continue
        assert rel_l2(a.numpy(), b.numpy()) < 1e-4, name
