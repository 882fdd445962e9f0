"""The real-scene (COLMAP) stage-2 path on the GPU against the reference's
own outputs (tests/golden/colmap_golden.npz, made by
tests/golden/make_colmap_golden.py) and the float64 oracle:

* the vertex frustum mask (in_frustum) for every screen piece — exact;
* the no-adjacency FlexiCubes on frustum cube subsets and on the whole
  grid without the C16/C19 re-check — faces and surface edges exact,
  vertices and L_dev within 2e-6, gradients 1e-4 relative L2 (float atomics);
* the real-scene binding (no scale factor) — means, covariances and vertex
  gradients as the stage-2 binding tests bound them;
* one per-view extraction as getMesh_in_frustum runs it: mask -> cubes ->
  extraction -> binding, for a screen half, against the oracle chain.
"""
import os

import numpy as np
import pytest
import torch

from dmgs_gb300.binding import bind_faces, vertex_frustum_mask
from dmgs_gb300.flexicubes import FlexiCubesNoAdjacent
from helpers import rel_l2
from oracle import binding as ob
from oracle import flexicubes as ofc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "colmap_golden.npz")
PIECES = [(-1, 0), (0, 2), (1, 2), (0, 4), (1, 4), (2, 4), (3, 4)]
D = "cuda"


@pytest.mark.parametrize("piece", PIECES)
def test_vertex_frustum_mask(piece):
    z = np.load(GOLDEN)
    m = vertex_frustum_mask(torch.tensor(z["verts"], device=D), torch.tensor(z["full_proj"], device=D),
                            float(z["cube_len"]), *piece)
    np.testing.assert_array_equal(m.cpu().numpy(), z[f"mask_{piece[0]}_{piece[1]}"])


def test_vertex_frustum_mask_and_mask():
    z = np.load(GOLDEN)
    rng = np.random.default_rng(0)
    extra = rng.random(z["verts"].shape[0]) < 0.5
    m = vertex_frustum_mask(torch.tensor(z["verts"], device=D), torch.tensor(z["full_proj"], device=D),
                            float(z["cube_len"]), 0, 2, and_mask=torch.tensor(extra, device=D))
    np.testing.assert_array_equal(m.cpu().numpy(), z["mask_0_2"] & extra)


@pytest.mark.parametrize("tag", ["view", "half", "quarter", "fullnoise"])
def test_no_adjacent_flexicubes_against_reference(tag):
    z = np.load(GOLDEN)
    res = tuple(int(r) for r in z["res"])
    fc = FlexiCubesNoAdjacent(device=D)
    if tag == "fullnoise":
        cubes = fc.construct_cubes(torch.ones(z["verts"].shape[0], dtype=torch.bool, device=D), res)
    else:
        key = {"view": "mask_-1_0", "half": "mask_1_2", "quarter": "mask_2_4"}[tag]
        cubes = fc.construct_cubes(torch.tensor(z[key], device=D), res)
    np.testing.assert_array_equal(cubes.cpu().numpy(), z[f"{tag}/cubes"])
    x = torch.tensor(z["x"], device=D, requires_grad=True)
    s = torch.tensor(z["noise"] if tag == "fullnoise" else z["s"], device=D, requires_grad=True)
    v, f, L, se = fc(x, s, cubes, res, training=bool(z[f"{tag}/training"]))
    np.testing.assert_array_equal(f.cpu().numpy(), z[f"{tag}/f"])
    np.testing.assert_array_equal(se.cpu().numpy(), z[f"{tag}/se"])
    np.testing.assert_allclose(v.detach().cpu().numpy(), z[f"{tag}/v"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(L.detach().cpu().numpy(), z[f"{tag}/L"], rtol=0, atol=2e-6)
    ((v * torch.tensor(z[f"{tag}/gv"], device=D)).sum()
     + (L * torch.tensor(z[f"{tag}/gl"], device=D)).sum()).backward()
    assert rel_l2(x.grad.cpu().numpy(), z[f"{tag}/dx"]) <= 1e-4
    assert rel_l2(s.grad.cpu().numpy(), z[f"{tag}/ds"]) <= 1e-4


def test_foreign_subset_tensor_is_recognised():
    """A cube list not made by this instance's construct_cubes (the
    reference's own tensor) is checked and used as a subset."""
    z = np.load(GOLDEN)
    res = tuple(int(r) for r in z["res"])
    fc = FlexiCubesNoAdjacent(device=D)
    x = torch.tensor(z["x"], device=D)
    s = torch.tensor(z["s"], device=D)
    v, f, L, se = fc(x, s, torch.tensor(z["half/cubes"], device=D), res, training=False)
    np.testing.assert_array_equal(f.cpu().numpy(), z["half/f"])
    with pytest.raises(NotImplementedError):
        fc(x, s, torch.tensor(z["half/cubes"][::-1].copy(), device=D), res)
    with pytest.raises(NotImplementedError):
        fc(x, s, torch.tensor(z["half/cubes"], device=D), res, de_ambiguity=True)


@pytest.mark.parametrize("G", [3, 6])
@pytest.mark.parametrize("adaptive", [True, False])
def test_binding_without_scale_factor_against_reference(G, adaptive):
    z = np.load(GOLDEN)
    tag = f"bind_G{G}_{'a' if adaptive else 'n'}"
    verts = torch.tensor(z["mesh_verts"], device=D, requires_grad=True)
    faces = torch.tensor(z["mesh_faces"], device=D)
    bc = torch.tensor(z[f"{tag}/bc"], device=D)
    xyz, cov, _ = bind_faces(verts, faces, bc, None, float(z[f"{tag}/rad"]), 2.5, adaptive_cov=adaptive)
    np.testing.assert_allclose(xyz.detach().cpu().numpy(), z[f"{tag}/xyz"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(cov.detach().cpu().numpy(), z[f"{tag}/cov"], rtol=1e-4,
                               atol=1e-5 * np.abs(z[f"{tag}/cov"]).max())
    ((xyz * torch.tensor(z[f"{tag}/gxyz"], device=D)).sum()
     + (cov * torch.tensor(z[f"{tag}/gcov"], device=D)).sum()).backward()
    assert rel_l2(verts.grad.cpu().numpy(), z[f"{tag}/dverts"]) <= 1e-4


def test_per_view_extraction_and_binding_against_oracle():
    """getMesh_in_frustum + renew_gaussian of the real-scene model for the
    right half of the screen: mask -> cube subset -> training-mode
    extraction -> binding without scale factor; means, covariances and the
    gradients w.r.t. the vertex positions and the field against the oracle
    chain in float64."""
    z = np.load(GOLDEN)
    res = tuple(int(r) for r in z["res"])
    fc = FlexiCubesNoAdjacent(device=D)
    grid = torch.tensor(z["verts"], device=D)
    m = vertex_frustum_mask(grid, torch.tensor(z["full_proj"], device=D), float(z["cube_len"]), 1, 2)
    cubes = fc.construct_cubes(m, res)
    x = torch.tensor(z["x"], device=D, requires_grad=True)
    s = torch.tensor(z["s"], device=D, requires_grad=True)
    v, f, L, se = fc(x, s, cubes, res, training=True)
    bc = torch.tensor(z["bind_G6_a/bc"], device=D)
    rad = float(z["bind_G6_a/rad"])
    xyz, cov, _ = bind_faces(v, f, bc, None, rad, 2.5)
    rng = np.random.default_rng(5)
    gx = rng.standard_normal(xyz.shape)
    gc = rng.standard_normal(cov.shape)
    ((xyz * torch.tensor(gx, device=D, dtype=torch.float32)).sum()
     + 1e3 * (cov * torch.tensor(gc, device=D, dtype=torch.float32)).sum()).backward()
    x64 = torch.tensor(z["x"], dtype=torch.float64, requires_grad=True)
    s64 = torch.tensor(z["s"], dtype=torch.float64, requires_grad=True)
    v64, f64, _, _ = ofc.extract(x64, s64, ofc.construct_cubes(z["mask_1_2"], res), res,
                                 training=True, de_ambiguity=False)
    np.testing.assert_array_equal(f.cpu().numpy(), f64.numpy())
    xr, cr, _, _ = ob.bind_stage2(v64, f64, torch.tensor(z["bind_G6_a/bc"], dtype=torch.float64),
                                  rad, 2.5e-6, None)
    np.testing.assert_allclose(xyz.detach().cpu().numpy(), xr.detach().numpy(), rtol=1e-5, atol=1e-5)
    ((xr * torch.tensor(gx)).sum() + 1e3 * (cr * torch.tensor(gc)).sum()).backward()
    assert rel_l2(x.grad.cpu().numpy(), x64.grad.numpy()) <= 1e-3
    assert rel_l2(s.grad.cpu().numpy(), s64.grad.numpy()) <= 1e-3
