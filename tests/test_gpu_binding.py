"""GPU parity of the face-binding kernels: against the reference's own
binding code (golden vectors) and against the FP64 oracle."""
import os

import numpy as np
import pytest
import torch

from dmgs_gb300.binding import barycentric_table, bind_faces, bind_faces_scale_rot
from helpers import rel_l2
from oracle import binding as OB

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("G", [1, 3, 6])
@pytest.mark.parametrize("adaptive", [True, False])
def test_stage2_against_reference(G, adaptive):
    z = np.load(os.path.join(GOLD, "binding_golden.npz"))
    tag = f"G{G}_{'a' if adaptive else 'n'}"
    d = "cuda"
    verts = torch.tensor(z["verts"], device=d, requires_grad=True)
    faces = torch.tensor(z["faces"], device=d)
    bc, rad = barycentric_table(G, d)
    np.testing.assert_allclose(bc.cpu().numpy(), z[f"{tag}_bc"], rtol=0, atol=1e-7)
    assert abs(rad - float(z[f"{tag}_rad"])) < 1e-9
    sf = torch.tensor([0.37], device=d, requires_grad=True)
    xyz, cov, covL = bind_faces(verts, faces, bc, sf, rad, 4.0, 2.0, adaptive)
    np.testing.assert_allclose(xyz.detach().cpu().numpy(), z[f"{tag}_xyz"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(cov.detach().cpu().numpy(), z[f"{tag}_cov"], rtol=1e-4, atol=1e-9)
    np.testing.assert_allclose(covL.cpu().numpy(), z[f"{tag}_covL"], rtol=1e-5, atol=1e-8)
    loss = (xyz * torch.tensor(z[f"{tag}_gxyz"], device=d)).sum() + \
           (cov * torch.tensor(z[f"{tag}_gcov"], device=d)).sum()
    loss.backward()
    assert rel_l2(verts.grad.cpu().numpy(), z[f"{tag}_dverts"]) <= 1e-4
    assert rel_l2(sf.grad.cpu().numpy(), z[f"{tag}_dsf"]) <= 1e-4


def test_stage2_per_gaussian_barycentrics_against_oracle():
    rng = np.random.default_rng(3)
    z = np.load(os.path.join(GOLD, "binding_golden.npz"))
    F = z["faces"].shape[0]
    bc = rng.dirichlet([1, 1, 1], (F, 6)).astype(np.float32)
    d = "cuda"
    verts = torch.tensor(z["verts"], device=d, requires_grad=True)
    sf = torch.tensor([0.2], device=d, requires_grad=True)
    _, rad = barycentric_table(6, d)
    xyz, cov, _ = bind_faces(verts, torch.tensor(z["faces"], device=d), torch.tensor(bc, device=d),
                             sf, rad, 4.0)
    v64 = torch.tensor(z["verts"], dtype=torch.float64, requires_grad=True)
    s64 = torch.tensor([0.2], dtype=torch.float64, requires_grad=True)
    x_ref, c_ref, _, _ = OB.bind_stage2(v64, torch.tensor(z["faces"]), torch.tensor(bc, dtype=torch.float64),
                                        rad, 4e-6, s64)
    np.testing.assert_allclose(xyz.detach().cpu().numpy(), x_ref.detach().numpy(), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(cov.detach().cpu().numpy(), c_ref.detach().numpy(), rtol=1e-4, atol=1e-9)
    gx = rng.standard_normal(xyz.shape)
    gc = rng.standard_normal(cov.shape)
    ((xyz * torch.tensor(gx, device=d, dtype=torch.float32)).sum()
     + (cov * torch.tensor(gc, device=d, dtype=torch.float32)).sum()).backward()
    ((x_ref * torch.tensor(gx)).sum() + (c_ref * torch.tensor(gc)).sum()).backward()
    assert rel_l2(verts.grad.cpu().numpy(), v64.grad.numpy()) <= 1e-4
    assert rel_l2(sf.grad.cpu().numpy(), s64.grad.numpy()) <= 1e-4


def _quat_to_R(q):
    r, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y),
                     2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x),
                     2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], 1).reshape(-1, 3, 3)


def test_stage3_against_reference_and_oracle():
    z = np.load(os.path.join(GOLD, "binding3_golden.npz"))
    d = "cuda"
    verts = torch.tensor(z["verts"], device=d, requires_grad=True)
    s2 = torch.tensor(z["scaling2d"], device=d, requires_grad=True)
    r2 = torch.tensor(z["rotation2d"], device=d, requires_grad=True)
    faces = torch.tensor(z["faces"], device=d)
    bc = torch.tensor(z["bc"], device=d)
    xyz, scales, rots = bind_faces_scale_rot(verts, faces, bc, s2, r2, float(z["thin_z"]))
    np.testing.assert_allclose(xyz.detach().cpu().numpy(), z["xyz"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(scales.detach().cpu().numpy(), z["scales"], rtol=1e-5, atol=1e-12)
    q = rots.detach().cpu().numpy()
    assert (q[:, 0] >= 0).all()
    np.testing.assert_allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-5)
    np.testing.assert_allclose(_quat_to_R(q), z["R"], atol=2e-5)
    # adjoint vs the FP64 oracle
    rng = np.random.default_rng(5)
    gx, gs, gq = (rng.standard_normal(t.shape) for t in (xyz, scales, rots))
    ((xyz * torch.tensor(gx, device=d, dtype=torch.float32)).sum()
     + (scales * torch.tensor(gs, device=d, dtype=torch.float32)).sum()
     + (rots * torch.tensor(gq, device=d, dtype=torch.float32)).sum()).backward()
    v64 = torch.tensor(z["verts"], dtype=torch.float64, requires_grad=True)
    s64 = torch.tensor(z["scaling2d"], dtype=torch.float64, requires_grad=True)
    r64 = torch.tensor(z["rotation2d"], dtype=torch.float64, requires_grad=True)
    x_o, sc_o, _, q_o = OB.bind_stage3(v64, torch.tensor(z["faces"]), torch.tensor(z["bc"], dtype=torch.float64),
                                       s64, r64, float(z["thin_z"]))
    np.testing.assert_allclose(q, q_o.detach().numpy(), atol=2e-5)
    ((x_o * torch.tensor(gx)).sum() + (sc_o * torch.tensor(gs)).sum() + (q_o * torch.tensor(gq)).sum()).backward()
    assert rel_l2(verts.grad.cpu().numpy(), v64.grad.numpy()) <= 1e-3
    assert rel_l2(s2.grad.cpu().numpy(), s64.grad.numpy()) <= 1e-4
    assert rel_l2(r2.grad.cpu().numpy(), r64.grad.numpy()) <= 1e-3


def test_frustum_face_culling_matches_the_reference_rule():
    import numpy as np
    from dmgs_gb300.binding import frustum_faces
    from dmgs_gb300.camera import make_view
    from dmgs_gb300.meshbound import sphere_torus_mesh
    v, f = sphere_torus_mesh(32)
    verts, faces = v.to("cuda"), f.to("cuda")
    view = make_view((1.2, 0.4, 1.0), (0.0, 0.0, 0.0), 200, 160, fovx_deg=40)
    M = torch.tensor(view.projmatrix, device="cuda")
    mask, kept, idx = frustum_faces(verts, faces, M)
    # the reference's in_frustum on face centroids, in float64
    c = verts.double()[faces].mean(dim=1)
    p = c @ M.double()[:3] + M.double()[3:]
    w = p[:, 3:] + 1e-6
    q = p[:, :3] / w
    ref = (q.abs() < 1.05).all(dim=-1) & (w.squeeze() > 0)
    near = ((q.abs() - 1.05).abs() < 1e-4).any(dim=-1) | (w.squeeze().abs() < 1e-4)
    assert torch.equal(mask[~near], ref[~near])
    assert 0 < int(mask.sum()) < len(f)
    assert torch.equal(idx, torch.nonzero(mask).squeeze(1))  # kept in face order
    assert torch.equal(kept, faces[mask])
    bad = faces.clone()
    bad[0, 0] = len(v) + 5  # out-of-range vertex: never kept
    m2, _, _ = frustum_faces(verts, bad, M)
    assert not bool(m2[0])


def test_frustum_face_culling_matches_reference_golden():
    """frustum_faces (dmgs_face_cull) against the masks of the reference's
    own in_frustum on face centroids (tests/golden/facecull_golden.npz),
    outside a 1e-4 band around the bounds (the oracle's margin), with the
    kept faces compacted in face order."""
    import os
    import numpy as np
    from dmgs_gb300.binding import frustum_faces
    from oracle import binding as ob
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "facecull_golden.npz"))
    verts = torch.tensor(z["verts"], device="cuda")
    faces = torch.tensor(z["faces"], device="cuda")
    c = z["verts"].astype(np.float64)[z["faces"]].mean(axis=1)
    for i in range(int(z["n"])):
        M = torch.tensor(z[f"proj{i}"], device="cuda")
        mask, kept, idx = frustum_faces(verts, faces, M)
        _, margin = ob.vertex_frustum_mask(c, z[f"proj{i}"], 0.0)
        ok = torch.tensor(margin.numpy() > 1e-4, device="cuda")
        ref = torch.tensor(z[f"mask{i}"], device="cuda")
        assert torch.equal(mask[ok], ref[ok])
        assert torch.equal(idx, torch.nonzero(mask).squeeze(1))
        assert torch.equal(kept, faces[mask])
