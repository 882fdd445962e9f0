"""Fused mesh -> Gaussian face binding (forward + adjoint) on the GPU.

* :func:`bind_faces` — stage-2 form, replacing the torch-op chain of
  ``renew_gaussian`` + ``get_covariance_dyn``
  (scene/gaussian_geo_model_mlp_flex.py:267-316, 370-385): returns the
  Gaussian means [F*G,3] and the shared per-face covariance [F*G,6]
  (``strip_symmetric`` packing); differentiable w.r.t. ``verts`` and
  ``scale_factor`` exactly like the reference (the triangle-space factor is
  a constant there, computed under ``torch.no_grad``).
* :func:`bind_faces_scale_rot` — stage-3 form
  (scene/gaussian_geo_model_finetune.py:414-421, 446-483): means, scales
  (exp of the 2D scale, thin z) and unit quaternions; differentiable w.r.t.
  ``verts``, the 2D scales and the 2D rotations.
"""
from __future__ import annotations

import math

import torch

from . import _lib
from ._lib import DmgsFaceBinding, DmgsFaceBinding3, check, ptr, stream_of


def barycentric_table(num, device="cuda"):
    """Shared barycentric coordinates and radius for 1, 3 or 6 Gaussians per
    face (the table of geo/mesh_utils.py:16-40)."""
    r3 = math.sqrt(3.0)
    if num == 1:
        bc, rad = [[1 / 3, 1 / 3, 1 / 3]], 1.0 / (2.0 * r3)
    elif num == 3:
        a, b = (3 - r3) / 6, r3 / 3
        bc, rad = [[a, a, b], [a, b, a], [b, a, a]], 1.0 / (2.0 + 2.0 * r3)
    elif num == 6:
        bc = [[2 / 3, 1 / 6, 1 / 6], [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3],
              [1 / 6, 5 / 12, 5 / 12], [5 / 12, 1 / 6, 5 / 12], [5 / 12, 5 / 12, 1 / 6]]
        rad = 1.0 / (4.0 + 2.0 * r3)
    else:
        raise NotImplementedError(num)
    return torch.tensor(bc, dtype=torch.float32, device=device), rad


def _prep(t, dtype=torch.float32):
    return t.detach().to(dtype=dtype).contiguous()


class _Bind2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, verts, scale_factor, faces, bc, G, per_g, rad_base, z_scale, max_scale,
                adaptive):
        lib = _lib.load()
        v = _prep(verts)
        f = faces.detach().to(torch.int64).contiguous()
        b = _prep(bc)
        sf = None if scale_factor is None else _prep(scale_factor).reshape(1)
        F = f.shape[0]
        desc = DmgsFaceBinding(F, v.shape[0], G, int(bool(per_g)), int(bool(adaptive)), float(rad_base), float(z_scale), float(max_scale),
                               ptr(v), ptr(f), ptr(b), ptr(sf))
        xyz = torch.empty(F * G, 3, device=v.device)
        cov = torch.empty(F * G, 6, device=v.device)
        covL = torch.empty(F, 3, 3, device=v.device)
        check(lib.dmgs_bind_fwd(desc, ptr(xyz), ptr(cov), None, ptr(covL), stream_of(v.device)),
              "bind_fwd")
        ctx.save_for_backward(v, f, b, sf)
        ctx.meta = (G, rad_base, z_scale, max_scale, adaptive, desc.bc_per_gaussian)
        ctx.sf_shape = None if scale_factor is None else tuple(scale_factor.shape)
        ctx.mark_non_differentiable(covL)
        return xyz, cov, covL

    @staticmethod
    def backward(ctx, dxyz, dcov, _dcovL):
        lib = _lib.load()
        v, f, b, sf = ctx.saved_tensors
        G, rad_base, z_scale, max_scale, adaptive, per_g = ctx.meta
        desc = DmgsFaceBinding(f.shape[0], v.shape[0], G, per_g, int(bool(adaptive)),
                               float(rad_base), float(z_scale), float(max_scale),
                               ptr(v), ptr(f), ptr(b), ptr(sf))
        dxyz = None if dxyz is None else _prep(dxyz)
        dcov = None if dcov is None else _prep(dcov)
        dverts = torch.empty_like(v)
        dsf = torch.empty(1, device=v.device) if sf is not None else None
        check(lib.dmgs_bind_bwd(desc, ptr(dxyz), ptr(dcov), ptr(dverts), ptr(dsf),
                                stream_of(v.device)), "bind_bwd")
        return (dverts, None if dsf is None else dsf.view(ctx.sf_shape), None, None, None, None,
                None, None, None, None)


def bind_faces(verts, faces, bc, scale_factor, rad_base, spatial_lr_scale, max_scale=2.0,
               adaptive_cov=True):
    """Stage-2 binding.  ``bc``: [G,3] shared table, or [F,G,3] per-Gaussian
    barycentric coordinates.  ``scale_factor``: the learnable scale of the
    synthetic-scene model (covariance factor tanh(scale_factor) * max_scale),
    or None for the real-scene model, whose covariance has no such factor
    (scene/gaussian_geo_model_mlp_flex_colmap.py:494-512).  Returns (xyz
    [F*G,3], covariance [F*G,6], cov3D_L [F,3,3])."""
    per_g = bc.dim() == 3
    G = bc.shape[1] if per_g else bc.shape[0]
    z_scale = float(spatial_lr_scale) * 1e-6
    return _Bind2.apply(verts, scale_factor, faces, bc.reshape(-1, 3), G, per_g, rad_base,
                        z_scale, max_scale, adaptive_cov)


class _Bind3(torch.autograd.Function):
    @staticmethod
    def forward(ctx, verts, scaling2d, rotation2d, faces, bc, thin_z):
        lib = _lib.load()
        v = _prep(verts)
        f = faces.detach().to(torch.int64).contiguous()
        b = _prep(bc)
        s2 = _prep(scaling2d)
        r2 = _prep(rotation2d)
        F, G = f.shape[0], b.shape[0]
        desc = DmgsFaceBinding3(F, v.shape[0], G, float(thin_z), ptr(v), ptr(f), ptr(b), ptr(s2),
                                ptr(r2))
        xyz = torch.empty(F * G, 3, device=v.device)
        scales = torch.empty(F * G, 3, device=v.device)
        rots = torch.empty(F * G, 4, device=v.device)
        check(lib.dmgs_bind3_fwd(desc, ptr(xyz), ptr(scales), ptr(rots), stream_of(v.device)),
              "bind3_fwd")
        ctx.save_for_backward(v, f, b, s2, r2)
        ctx.thin_z = thin_z
        return xyz, scales, rots

    @staticmethod
    def backward(ctx, dxyz, dscales, drots):
        lib = _lib.load()
        v, f, b, s2, r2 = ctx.saved_tensors
        desc = DmgsFaceBinding3(f.shape[0], v.shape[0], b.shape[0], float(ctx.thin_z), ptr(v),
                                ptr(f), ptr(b), ptr(s2), ptr(r2))
        dverts = torch.empty_like(v)
        ds2 = torch.empty_like(s2)
        dr2 = torch.empty_like(r2)
        check(lib.dmgs_bind3_bwd(desc, ptr(None if dxyz is None else _prep(dxyz)),
                                 ptr(None if dscales is None else _prep(dscales)),
                                 ptr(None if drots is None else _prep(drots)),
                                 ptr(dverts), ptr(ds2), ptr(dr2), stream_of(v.device)), "bind3_bwd")
        return dverts, ds2, dr2, None, None, None


def bind_faces_scale_rot(verts, faces, bc, scaling2d, rotation2d, thin_z):
    """Stage-3 binding.  Returns (xyz, scales, rotations) for the rasteriser's
    scale/rotation input mode."""
    return _Bind3.apply(verts, scaling2d, rotation2d, faces, bc, thin_z)


def frustum_faces(verts, faces, full_proj):
    """Stage-3 frustum face selection (scene/gaussian_geo_model_finetune.py:
    33-48,404-409): the faces whose centroid lies inside 1.05x the clip volume
    of the camera's full_proj_transform (stored [4,4], row-vector
    convention).  Returns (face_mask bool [F], kept faces [F',3] int64, kept
    face indices [F'] int64); the reference's gs_mask is
    face_mask.repeat_interleave(G)."""
    lib = _lib.load()
    v = _prep(verts)
    f = faces.detach().to(torch.int64).contiguous()
    M = _prep(full_proj)
    F = f.shape[0]
    dev = v.device
    mask = torch.empty(F, dtype=torch.uint8, device=dev)
    kept = torch.empty(max(F, 1), dtype=torch.int32, device=dev)
    num = torch.zeros(1, dtype=torch.int32, device=dev)
    scratch = torch.empty(max(int(lib.dmgs_face_cull_scratch_bytes(F)), 1), dtype=torch.uint8,
                          device=dev)
    check(lib.dmgs_face_cull(ptr(v), v.shape[0], ptr(f), F, ptr(M), ptr(mask), ptr(kept), ptr(num),
                             ptr(scratch), scratch.numel(), stream_of(dev)), "face_cull")
    idx = kept[:int(num.item())].long()
    return mask.bool(), f[idx], idx


def vertex_frustum_mask(verts, full_proj, cube_len, piece_id=-1, n_piece=0, and_mask=None):
    """The real-scene stage 2's vertex frustum mask (in_frustum,
    scene/gaussian_geo_model_mlp_flex_colmap.py:31-76): grid vertices moved
    by half a cube edge, taken through the camera's full_proj_transform
    (stored [4,4]) and kept inside the whole screen (piece_id < 0), one half
    (n_piece 2) or one quarter (n_piece 4) of it, widened by 0.05; and_mask
    (bool [N], the background grid's vertex mask) is ANDed in.  Returns a
    bool [N] mask for FlexiCubesNoAdjacent.construct_cubes."""
    lib = _lib.load()
    v = _prep(verts)
    M = _prep(full_proj)
    N = v.shape[0]
    out = torch.empty(N, dtype=torch.uint8, device=v.device)
    am = None if and_mask is None else and_mask.reshape(-1).to(torch.uint8).contiguous()
    check(lib.dmgs_vertex_frustum_mask(ptr(v), N, ptr(M), float(cube_len), int(piece_id),
                                       int(n_piece), ptr(am), ptr(out), stream_of(v.device)),
          "vertex_frustum_mask")
    return out.bool()
