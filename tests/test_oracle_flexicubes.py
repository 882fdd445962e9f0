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
REF_TABLES = "/root/reference/geo/tables.py"
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
    if not os.path.exists(REF_TABLES):
        pytest.skip("reference tree not present")
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
