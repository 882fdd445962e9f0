"""CPU oracle of the mesh -> Gaussian face binding — TEST INFRASTRUCTURE ONLY.

FP64 torch restatement (autograd gives the adjoint) of

* stage 2: ``renew_gaussian`` (scene/gaussian_geo_model_mlp_flex.py:258-335)
  and ``get_covariance_dyn`` (:370-385), with ``face_normals``
  (geo/mesh_utils.py:43-57) and ``generate_barycentric_v2`` (:16-40);
* stage 3: ``renew_gaussian`` (scene/gaussian_geo_model_finetune.py:396-421),
  ``get_scaling`` (:446-454), ``get_rot_matrix`` (:465-483) and
  ``get_rotation`` (:456-463), whose matrix->quaternion step (pytorch3d's
  ``matrix_to_quaternion``, absent here) is restated as Shepperd's method
  with a non-negative real part.

Pinned against the reference's own code by ``tests/golden/binding*_golden.npz``.
"""
from __future__ import annotations

import math

import torch

EPS = 1e-12


def barycentric_table(num):
    """Barycentric coordinates and std-dev radius of generate_barycentric_v2
    (geo/mesh_utils.py:16-40) for 1, 3 or 6 Gaussians per face."""
    r3 = math.sqrt(3.0)
    if num == 1:
        return torch.tensor([[1 / 3, 1 / 3, 1 / 3]], dtype=torch.float64), 1.0 / (2.0 * r3)
    if num == 3:
        a, b = (3 - r3) / 6, r3 / 3
        return torch.tensor([[a, a, b], [a, b, a], [b, a, a]], dtype=torch.float64), 1.0 / (2.0 + 2.0 * r3)
    if num == 6:
        return torch.tensor([[2 / 3, 1 / 6, 1 / 6], [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3],
                             [1 / 6, 5 / 12, 5 / 12], [5 / 12, 1 / 6, 5 / 12], [5 / 12, 5 / 12, 1 / 6]],
                            dtype=torch.float64), 1.0 / (4.0 + 2.0 * r3)
    raise NotImplementedError(num)


def _unit(v):
    return v / v.norm(dim=-1, keepdim=True).clamp_min(EPS)


def face_frames(verts, faces):
    tri = verts[faces]                         # [F,3,3]
    e01 = tri[:, 1] - tri[:, 0]
    e02 = tri[:, 2] - tri[:, 0]
    x = _unit(e01)
    n = _unit(torch.cross(e01, e02, dim=-1))
    y = _unit(torch.cross(n, x, dim=-1))
    R = torch.stack([x, y, n], dim=2)          # columns x, y, n
    return tri, e01, e02, x, y, n, R


def bind_stage2(verts, faces, bc, rad_base, z_scale, scale_factor, max_scale=2.0,
                adaptive=True):
    """Returns xyz [F*G,3], cov [F*G,6], R [F,3,3], covL [F,3,3].  `bc` is
    [G,3] (shared) or [F,G,3] (per Gaussian); scale_factor None: no
    covariance factor (the real-scene model)."""
    tri, e01, e02, x, y, n, R = face_frames(verts, faces)
    F = faces.shape[0]
    if bc.dim() == 2:
        xyz = torch.einsum("gk,fkc->fgc", bc, tri)
    else:
        xyz = torch.einsum("fgk,fkc->fgc", bc, tri)
    G = xyz.shape[1]
    xyz = xyz.reshape(-1, 3)
    with torch.no_grad():
        ln = e01.norm(dim=-1).clamp_min(EPS)
        if adaptive:
            Ax = (e02 * x).sum(-1)
            Ay = (e02 * y).sum(-1)
            Ex, Ey = ln / 2.0, ln * (math.sqrt(3.0) / 2.0)
            m01 = (Ax - Ex) / Ey
            m11 = Ay / Ey
        else:
            m01 = torch.zeros_like(ln)
            m11 = torch.ones_like(ln)
        s = ln * rad_base
        L = torch.zeros(F, 3, 3, dtype=verts.dtype)
        L[:, 0, 0] = s
        L[:, 0, 1] = m01 * s
        L[:, 1, 1] = m11 * s
        L[:, 2, 2] = z_scale
    # no scale factor: the real-scene model (scene/gaussian_geo_model_mlp_flex_colmap.py:494-512)
    k = torch.tanh(scale_factor) * max_scale if scale_factor is not None else 1.0
    M = R @ (L * k)
    S = M @ M.transpose(1, 2)
    c6 = torch.stack([S[:, 0, 0], S[:, 0, 1], S[:, 0, 2], S[:, 1, 1], S[:, 1, 2], S[:, 2, 2]], 1)
    cov = c6.view(F, 1, 6).expand(F, G, 6).reshape(-1, 6)
    return xyz, cov, R, L


def quat_from_matrix(R):
    """Unit quaternion (w, x, y, z), w >= 0, of rotation matrices [N,3,3]
    by Shepperd's method: divide by the largest of 4w^2, 4x^2, 4y^2, 4z^2."""
    m00, m01, m02 = R[:, 0, 0], R[:, 0, 1], R[:, 0, 2]
    m10, m11, m12 = R[:, 1, 0], R[:, 1, 1], R[:, 1, 2]
    m20, m21, m22 = R[:, 2, 0], R[:, 2, 1], R[:, 2, 2]
    tr = m00 + m11 + m22
    args = torch.stack([1 + tr, 1 + m00 - m11 - m22, 1 - m00 + m11 - m22, 1 - m00 - m11 + m22], 1)
    big = 0.5 * args.clamp_min(0).sqrt()
    d = 0.25 / big.clamp_min(0.05)
    cand = torch.stack([
        torch.stack([big[:, 0], (m21 - m12) * d[:, 0], (m02 - m20) * d[:, 0], (m10 - m01) * d[:, 0]], 1),
        torch.stack([(m21 - m12) * d[:, 1], big[:, 1], (m01 + m10) * d[:, 1], (m02 + m20) * d[:, 1]], 1),
        torch.stack([(m02 - m20) * d[:, 2], (m01 + m10) * d[:, 2], big[:, 2], (m12 + m21) * d[:, 2]], 1),
        torch.stack([(m10 - m01) * d[:, 3], (m02 + m20) * d[:, 3], (m12 + m21) * d[:, 3], big[:, 3]], 1),
    ], 1)                                        # [N, 4 branches, 4]
    with torch.no_grad():
        br = torch.stack([tr, m00, m11, m22], 1)
        # ties resolved in the order trace, m00, m11, m22
        choice = torch.where(
            (tr >= m00) & (tr >= m11) & (tr >= m22), torch.zeros_like(tr, dtype=torch.long),
            torch.where((m00 >= m11) & (m00 >= m22), torch.ones_like(tr, dtype=torch.long),
                        torch.where(m11 >= m22, torch.full_like(tr, 2, dtype=torch.long),
                                    torch.full_like(tr, 3, dtype=torch.long))))
        del br
    q = cand[torch.arange(R.shape[0]), choice]
    q = torch.where(q[:, :1] < 0, -q, q)
    return _unit(q)


def bind_stage3(verts, faces, bc, scaling2d, rotation2d, thin_z):
    """Returns xyz [F*G,3], scales [F*G,3], R [F*G,3,3], quaternions [F*G,4]."""
    tri, e01, e02, x, y, n, Rw = face_frames(verts, faces)
    G = bc.shape[0]
    xyz = torch.einsum("gk,fkc->fgc", bc, tri).reshape(-1, 3)
    scales = torch.cat([torch.exp(scaling2d), torch.full_like(scaling2d[:, :1], thin_z)], 1)
    c = _unit(rotation2d)
    Rt = torch.zeros(c.shape[0], 3, 3, dtype=c.dtype)
    Rt[:, 0, 0] = c[:, 0]
    Rt[:, 0, 1] = -c[:, 1]
    Rt[:, 1, 0] = c[:, 1]
    Rt[:, 1, 1] = c[:, 0]
    Rt[:, 2, 2] = 1.0
    R = (Rw.view(-1, 1, 3, 3) @ Rt.view(-1, G, 3, 3)).view(-1, 3, 3)
    return xyz, scales, R, quat_from_matrix(R)


def vertex_frustum_mask(verts, full_proj, cube_len, piece_id=-1, n_piece=0):
    """The real-scene stage 2's vertex frustum test (``in_frustum``,
    scene/gaussian_geo_model_mlp_flex_colmap.py:31-76) in float64: vertices
    moved by half a cube edge through full_proj (row-vector convention,
    stored [4,4]); kept when w = p.w + 1e-6 > 0 and p.xyz / w lies in the
    screen piece widened by 0.05 (whole screen, halves left / right,
    quarters bit 0 right, bit 1 top).  Returns (mask bool [N], margin [N]:
    the distance of the deciding coordinate to its bound, for the tests'
    float32 ambiguity band)."""
    v = torch.as_tensor(verts, dtype=torch.float64) + cube_len / 2.0
    M = torch.as_tensor(full_proj, dtype=torch.float64).reshape(4, 4)
    p = v @ M[:3] + M[3]
    w = p[:, 3] + 1e-6
    q = p[:, :3] / w.unsqueeze(1)
    lo = torch.tensor([-1.0, -1.0, -1.0], dtype=torch.float64)
    hi = torch.tensor([1.0, 1.0, 1.0], dtype=torch.float64)
    if piece_id >= 0:
        if n_piece == 2:
            (hi if piece_id == 0 else lo)[0] = 0.0
        elif n_piece == 4:
            (lo if piece_id & 1 else hi)[0] = 0.0
            (lo if piece_id & 2 else hi)[1] = 0.0
        else:
            raise NotImplementedError(n_piece)
    d = torch.minimum(q - (lo - 0.05), (hi + 0.05) - q)
    mask = (d > 0).all(1) & (w > 0)
    margin = torch.minimum(d.abs().min(1).values, w.abs())
    return mask, margin
