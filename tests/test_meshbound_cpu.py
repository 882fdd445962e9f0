"""The configuration-2 mesh: FlexiCubes' training-mode face count of the
sphere-union-torus field (45,304 at 64^3), closed, consistently outward."""
import numpy as np

from dmgs_gb300.meshbound import eval_sh, sdf_sphere_torus, sphere_torus_mesh


def test_sphere_torus_mesh_is_closed_outward_with_the_reference_face_count():
    v, f = sphere_torus_mesh(64)
    assert f.shape == (45304, 3) and f.min() >= 0 and f.max() < len(v)
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert np.all(counts == 2)  # every edge shared by exactly two faces
    c = v[f].mean(1)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    h = 1e-3
    grad = np.stack([(sdf_sphere_torus(c + h * np.eye(3)[i]) - sdf_sphere_torus(c - h * np.eye(3)[i]))
                     / (2 * h) for i in range(3)], 1)
    assert np.all((n * grad).sum(1) > 0)
    assert np.abs(sdf_sphere_torus(v)).max() < 2.0 / 64


def test_eval_sh_matches_the_oracle_polynomial():
    import torch
    from oracle import raster as R
    rng = np.random.default_rng(0)
    sh = rng.normal(0, 0.3, (50, 16, 3)).astype(np.float32)
    d = rng.normal(size=(50, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ours = eval_sh(3, torch.tensor(sh).permute(0, 2, 1), torch.tensor(d, dtype=torch.float32)).numpy()
    ref = R.eval_sh_rgb(3, sh.astype(np.float64), d)
    assert np.abs(ours + 0.5 - ref).max() < 1e-5  # the oracle adds the rasteriser offset
