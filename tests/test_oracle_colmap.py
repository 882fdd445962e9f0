"""The real-scene (COLMAP) stage-2 oracle pinned to the reference (CPU).

tests/golden/colmap_golden.npz holds outputs of the reference's own code
(tests/golden/make_colmap_golden.py): in_frustum masks for every screen
piece, the no-adjacency FlexiCubes on frustum cube subsets and on the whole
grid (no C16/C19 re-check), and renew_gaussian / get_covariance_dyn of the
real-scene model.  Bars: masks and integer outputs exact; float outputs to
float32 rounding (the oracle runs in float64); gradients 1e-5 relative L2.
"""
import os

import numpy as np
import pytest
import torch

from oracle import binding as ob
from oracle import flexicubes as ofc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "colmap_golden.npz")
PIECES = [(-1, 0), (0, 2), (1, 2), (0, 4), (1, 4), (2, 4), (3, 4)]


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("piece", PIECES)
def test_vertex_frustum_mask_matches_reference(piece):
    z = np.load(GOLDEN)
    m, margin = ob.vertex_frustum_mask(z["verts"], z["full_proj"], float(z["cube_len"]), *piece)
    ref = z[f"mask_{piece[0]}_{piece[1]}"]
    assert margin.min() > 1e-6  # no vertex in float32's ambiguity band
    np.testing.assert_array_equal(m.numpy(), ref)
    assert 0 < ref.sum() < ref.size


def test_construct_cubes_matches_reference():
    z = np.load(GOLDEN)
    res = tuple(int(r) for r in z["res"])
    np.testing.assert_array_equal(ofc.construct_cubes(z["mask_-1_0"], res).numpy(), z["view/cubes"])
    np.testing.assert_array_equal(ofc.construct_cubes(z["mask_1_2"], res).numpy(), z["half/cubes"])


@pytest.mark.parametrize("tag", ["view", "half", "quarter", "fullnoise"])
def test_no_adjacent_flexicubes_matches_reference(tag):
    z = np.load(GOLDEN)
    res = tuple(int(r) for r in z["res"])
    x = torch.tensor(z["x"], dtype=torch.float64, requires_grad=True)
    s = torch.tensor(z["noise"] if tag == "fullnoise" else z["s"], dtype=torch.float64,
                     requires_grad=True)
    v, f, L, se = ofc.extract(x, s, torch.tensor(z[f"{tag}/cubes"]), res,
                              training=bool(z[f"{tag}/training"]), de_ambiguity=False)
    np.testing.assert_array_equal(f.numpy(), z[f"{tag}/f"])
    np.testing.assert_array_equal(se.numpy(), z[f"{tag}/se"])
    np.testing.assert_allclose(v.detach().numpy(), z[f"{tag}/v"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(L.detach().numpy(), z[f"{tag}/L"], rtol=0, atol=2e-6)
    ((v * torch.tensor(z[f"{tag}/gv"], dtype=torch.float64)).sum()
     + (L * torch.tensor(z[f"{tag}/gl"], dtype=torch.float64)).sum()).backward()
    assert rel_l2(x.grad, z[f"{tag}/dx"]) <= 1e-5
    assert rel_l2(s.grad, z[f"{tag}/ds"]) <= 1e-5


@pytest.mark.parametrize("G", [3, 6])
@pytest.mark.parametrize("adaptive", [True, False])
def test_binding_without_scale_factor_matches_reference(G, adaptive):
    z = np.load(GOLDEN)
    tag = f"bind_G{G}_{'a' if adaptive else 'n'}"
    v = torch.tensor(z["mesh_verts"], dtype=torch.float64, requires_grad=True)
    xyz, cov, _, _ = ob.bind_stage2(v, torch.tensor(z["mesh_faces"]),
                                    torch.tensor(z[f"{tag}/bc"], dtype=torch.float64),
                                    float(z[f"{tag}/rad"]), 2.5e-6, None, adaptive=adaptive)
    np.testing.assert_allclose(xyz.detach().numpy(), z[f"{tag}/xyz"], rtol=1e-6, atol=1e-7)
    # entries that cancel to near zero carry float32 rounding of the largest ones
    np.testing.assert_allclose(cov.detach().numpy(), z[f"{tag}/cov"], rtol=1e-5,
                               atol=1e-5 * np.abs(z[f"{tag}/cov"]).max())
    ((xyz * torch.tensor(z[f"{tag}/gxyz"], dtype=torch.float64)).sum()
     + (cov * torch.tensor(z[f"{tag}/gcov"], dtype=torch.float64)).sum()).backward()
    assert rel_l2(v.grad, z[f"{tag}/dverts"]) <= 1e-5


def test_face_culling_rule_matches_reference_in_frustum():
    """The stage-3 face culling rule (in_frustum on face centroids,
    scene/gaussian_geo_model_finetune.py:33-48 as renew_gaussian applies it,
    :405-409) — the oracle's frustum test with no half-cube shift on the
    centroids — against golden masks from the reference's own function
    (tests/golden/make_facecull_golden.py), outside a 1e-4 band around the
    bounds where float32 and float64 may decide differently."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "facecull_golden.npz"))
    c = z["verts"].astype(np.float64)[z["faces"]].mean(axis=1)
    for i in range(int(z["n"])):
        m, margin = ob.vertex_frustum_mask(c, z[f"proj{i}"], 0.0)
        ok = margin.numpy() > 1e-4
        assert ok.mean() > 0.99
        assert np.array_equal(m.numpy()[ok], z[f"mask{i}"][ok])
        assert 0 < z[f"mask{i}"].sum() < len(z["faces"])
