"""CPU oracle of the differentiable Gaussian rasteriser — TEST INFRASTRUCTURE ONLY.

PARITY UNPINNED for the rasteriser core: the reference's rasteriser is the
un-vendored submodule graphdeco-inria/diff-gaussian-rasterization (unknown
commit, ``.gitmodules:4-6``), called from ``gaussian_renderer/__init__.py:86-94``.
This module restates the published 3DGS algorithm (Kerbl et al. 2023) with
EWA splatting (Zwicker et al. 2002); the reference-tree conventions it relies
on are pinned by ``tests/golden``.

Two halves:

``geometry_f32``  numpy float32 emulation of the per-Gaussian geometry stage in
    the exact operation order the CUDA kernel uses (separate IEEE mul/add,
    correctly rounded div/sqrt, no FMA).  Everything that decides an integer
    (cull, radius, tile rectangle, depth key) is computed here, so radii,
    ``tiles_touched``, sorted keys/values and tile ranges must match the
    kernel bit for bit.

``render``        FP64 torch restatement of the continuous part: projection,
    covariance, conic, SH colour and front-to-back blending, on the tile
    lists of the FP32 stage.  Its autograd backward reproduces the reference
    adjoint's conventions:
      * alpha = min(0.99, o*G) back-propagates as o*G (the cap is not
        differentiated);
      * the 1.3*tan(fov) clamp of the projected position inside the EWA
        Jacobian has zero gradient w.r.t. the clamped coordinate and treats
        the clamped value as a constant;
      * the screen-space-mean gradient is reported w.r.t. NDC (x, y)
        (pixel = ((ndc+1)*S-1)/2), the quantity the reference's
        densification consumes (``scene/gaussian_model.py:405-406``);
      * the quaternion is used as given (not normalised).
    Pixels whose result hinges on a threshold test that FP32 cannot decide
    are reported in ``ambiguous``: alpha within a relative band of 1/255 (the
    larger of 1e-5 and the exponent's FP32 reach: 4 ulp of the projected
    mean's pixel coordinates times the exponent's derivative w.r.t. the
    mean, plus 4 ulp of its terms), or transmittance within a relative band
    of 1e-4 (1e-5 plus the bands of the alphas blended before it).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

F32 = np.float32
BLOCK = 16

SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005,
         -1.0925484305920792, 0.5462742152960396)
SH_C3 = (-0.5900435899266435, 2.890611442640554, -0.4570457994644658,
         0.3731763325901154, -0.4570457994644658, 1.445305721320277,
         -0.5900435899266435)


@dataclass
class Camera:
    """Per-view constants, the fields of ``GaussianRasterizationSettings``
    (built at ``gaussian_renderer/__init__.py:36-49``).  ``viewmatrix`` and
    ``projmatrix`` are 4x4 in the reference's transposed (row-vector) storage
    (``scene/cameras.py:54-56``); flattened row-major they are the
    column-major matrices the kernel indexes."""
    width: int
    height: int
    tanfovx: float
    tanfovy: float
    viewmatrix: np.ndarray
    projmatrix: np.ndarray
    campos: np.ndarray
    bg: np.ndarray
    scale_modifier: float = 1.0
    sh_degree: int = 3
    prefiltered: bool = False

    @property
    def grid(self):
        return ((self.width + BLOCK - 1) // BLOCK, (self.height + BLOCK - 1) // BLOCK)


def _trunc_int(v: np.ndarray) -> np.ndarray:
    """float32 -> int32 truncation with the kernel's saturating semantics
    (``cvt.rzi.s32.f32``: NaN -> 0, out-of-range -> INT_MIN/INT_MAX)."""
    d = np.trunc(v.astype(np.float64))
    d = np.where(np.isnan(d), 0.0, d)
    return np.clip(d, -2147483648.0, 2147483647.0).astype(np.int64)


def focal(cam: Camera):
    """focal = size / (2 * tan(fov/2)) in float32, computed once per view."""
    fx = F32(cam.width) / (F32(2.0) * F32(cam.tanfovx))
    fy = F32(cam.height) / (F32(2.0) * F32(cam.tanfovy))
    return F32(fx), F32(fy)


def cov3d_from_scale_rot_f32(scales, rots, mod):
    """Sigma = R S S^T R^T, S = diag(mod*scale), R from the (unnormalised)
    quaternion (r, x, y, z) as in ``utils/general_utils.py:78-110``.
    Returns the 6-float upper-triangle packing of ``strip_lowerdiag``
    (``utils/general_utils.py:64-73``)."""
    mod = F32(mod)
    s = scales.astype(F32) * mod
    r, x, y, z = (rots[:, i].astype(F32) for i in range(4))
    one, two = F32(1), F32(2)
    R = np.empty((len(s), 3, 3), F32)
    R[:, 0, 0] = one - two * (y * y + z * z)
    R[:, 0, 1] = two * (x * y - r * z)
    R[:, 0, 2] = two * (x * z + r * y)
    R[:, 1, 0] = two * (x * y + r * z)
    R[:, 1, 1] = one - two * (x * x + z * z)
    R[:, 1, 2] = two * (y * z - r * x)
    R[:, 2, 0] = two * (x * z - r * y)
    R[:, 2, 1] = two * (y * z + r * x)
    R[:, 2, 2] = one - two * (x * x + y * y)
    M = R * s[:, None, :]
    def sig(i, k):
        return (M[:, i, 0] * M[:, k, 0] + M[:, i, 1] * M[:, k, 1]) + M[:, i, 2] * M[:, k, 2]
    return np.stack([sig(0, 0), sig(0, 1), sig(0, 2), sig(1, 1), sig(1, 2), sig(2, 2)], 1)


def geometry_f32(means3D, cam: Camera, opacities, scales=None, rotations=None, cov3D=None):
    """FP32 emulation of the preprocess stage (integer-determining part).

    Order of operations (shared with ``preprocess`` in the CUDA source):
      view  = ((V0*x + V4*y) + V8*z) + V12      (V column-major)
      cull  if view.z <= 0.2
      hom   = ((P0*x + P4*y) + P8*z) + P12, ... w with P3,P7,P11,P15
      ndc   = hom.xy * (1 / (hom.w + 1e-7))
      pix   = ((ndc + 1) * size - 1) * 0.5
      EWA   txtz = vx/vz clamped to +-1.3 tanfov, J = [[fx/vz, 0, -(fx*tx)/(vz*vz)],
            [0, fy/vz, -(fy*ty)/(vz*vz)]], T = J W, cov2 = T Sigma T^T, +0.3 on the diagonal
      cull  if det == 0; conic = (c11, -c01, c00) / det
      rad   = ceil(3 sqrt(mid + sqrt(max(0.1, mid^2 - det)))), mid = (c00+c11)/2
      rect  min = clamp(trunc((pix - rad)/16), 0, grid), max = clamp(trunc(((pix + rad) + 15)/16), 0, grid)
      cull  if rad <= 0 or the rectangle is empty
    """
    P = means3D.shape[0]
    m = means3D.astype(F32)
    x, y, z = m[:, 0], m[:, 1], m[:, 2]
    V = np.asarray(cam.viewmatrix, F32).reshape(16)
    Pm = np.asarray(cam.projmatrix, F32).reshape(16)
    vx = ((V[0] * x + V[4] * y) + V[8] * z) + V[12]
    vy = ((V[1] * x + V[5] * y) + V[9] * z) + V[13]
    vz = ((V[2] * x + V[6] * y) + V[10] * z) + V[14]
    front = vz > F32(0.2)
    hx = ((Pm[0] * x + Pm[4] * y) + Pm[8] * z) + Pm[12]
    hy = ((Pm[1] * x + Pm[5] * y) + Pm[9] * z) + Pm[13]
    hw = ((Pm[3] * x + Pm[7] * y) + Pm[11] * z) + Pm[15]
    with np.errstate(all="ignore"):
        pw = F32(1) / (hw + F32(1e-7))
        ndcx = hx * pw
        ndcy = hy * pw
        Wf, Hf = F32(cam.width), F32(cam.height)
        px = ((ndcx + F32(1)) * Wf - F32(1)) * F32(0.5)
        py = ((ndcy + F32(1)) * Hf - F32(1)) * F32(0.5)

        if cov3D is None:
            cov = cov3d_from_scale_rot_f32(scales, rotations, cam.scale_modifier)
        else:
            cov = cov3D.astype(F32)
        S00, S01, S02, S11, S12, S22 = (cov[:, i] for i in range(6))
        Sg = [[S00, S01, S02], [S01, S11, S12], [S02, S12, S22]]

        fx, fy = focal(cam)
        limx = F32(1.3) * F32(cam.tanfovx)
        limy = F32(1.3) * F32(cam.tanfovy)
        txtz = vx / vz
        tytz = vy / vz
        tx = np.minimum(limx, np.maximum(-limx, txtz)) * vz
        ty = np.minimum(limy, np.maximum(-limy, tytz)) * vz
        vz2 = vz * vz
        J00 = fx / vz
        J02 = -(fx * tx) / vz2
        J11 = fy / vz
        J12 = -(fy * ty) / vz2
        W = [[V[0], V[4], V[8]], [V[1], V[5], V[9]], [V[2], V[6], V[10]]]
        T0 = [J00 * W[0][j] + J02 * W[2][j] for j in range(3)]
        T1 = [J11 * W[1][j] + J12 * W[2][j] for j in range(3)]
        U0 = [(T0[0] * Sg[0][j] + T0[1] * Sg[1][j]) + T0[2] * Sg[2][j] for j in range(3)]
        U1 = [(T1[0] * Sg[0][j] + T1[1] * Sg[1][j]) + T1[2] * Sg[2][j] for j in range(3)]
        c00 = (U0[0] * T0[0] + U0[1] * T0[1]) + U0[2] * T0[2]
        c01 = (U0[0] * T1[0] + U0[1] * T1[1]) + U0[2] * T1[2]
        c11 = (U1[0] * T1[0] + U1[1] * T1[1]) + U1[2] * T1[2]
        c00 = c00 + F32(0.3)
        c11 = c11 + F32(0.3)
        det = c00 * c11 - c01 * c01
        det_ok = det != F32(0)
        det_inv = F32(1) / det
        conic = np.stack([c11 * det_inv, -c01 * det_inv, c00 * det_inv], 1)
        mid = F32(0.5) * (c00 + c11)
        disc = np.maximum(F32(0.1), mid * mid - det)
        sq = np.sqrt(disc)
        l1 = mid + sq
        l2 = mid - sq
        radf = np.ceil(F32(3) * np.sqrt(np.maximum(l1, l2)))
        rad = _trunc_int(radf)

        gx, gy = cam.grid
        r = rad.astype(F32)
        rminx = np.minimum(gx, np.maximum(0, _trunc_int((px - r) / F32(BLOCK))))
        rminy = np.minimum(gy, np.maximum(0, _trunc_int((py - r) / F32(BLOCK))))
        rmaxx = np.minimum(gx, np.maximum(0, _trunc_int(((px + r) + F32(BLOCK - 1)) / F32(BLOCK))))
        rmaxy = np.minimum(gy, np.maximum(0, _trunc_int(((py + r) + F32(BLOCK - 1)) / F32(BLOCK))))
    area = (rmaxx - rminx) * (rmaxy - rminy)
    visible = front & det_ok & (rad > 0) & (area > 0)
    radii = np.where(visible, rad, 0).astype(np.int32)
    tiles = np.where(visible, area, 0).astype(np.uint32)
    rect = np.stack([rminx, rminy, rmaxx, rmaxy], 1).astype(np.int64)
    depth = vz.astype(F32)
    return dict(radii=radii, tiles_touched=tiles, rect=rect, depth=depth,
                xy=np.stack([px, py], 1).astype(F32), conic=conic.astype(F32),
                visible=visible, prefilter_violation=bool(cam.prefiltered and (~front).any()))


def binning(geom, cam: Camera):
    """Tile binning: one instance per (visible Gaussian, touched tile) with key
    ``(tile << 32) | float_bits(depth)`` and value = Gaussian index, sorted by
    key; ties keep Gaussian-index order (a stable sort of the instance list
    emitted in Gaussian order).  Returns (keys u64 [K], values u32 [K],
    ranges u32 [T,2]); tiles with no instance have range (0, 0)."""
    gx, gy = cam.grid
    T = gx * gy
    vis = np.nonzero(geom["visible"])[0]
    rect = geom["rect"][vis]
    dbits = geom["depth"][vis].view(np.uint32).astype(np.uint64)
    tiles_l, ids_l, db_l = [], [], []
    for k in range(len(vis)):
        x0, y0, x1, y1 = rect[k]
        ys, xs = np.meshgrid(np.arange(y0, y1), np.arange(x0, x1), indexing="ij")
        t = (ys * gx + xs).reshape(-1)
        tiles_l.append(t)
        ids_l.append(np.full(t.shape, vis[k], np.int64))
        db_l.append(np.full(t.shape, dbits[k], np.uint64))
    if tiles_l:
        tiles = np.concatenate(tiles_l).astype(np.uint64)
        ids = np.concatenate(ids_l)
        db = np.concatenate(db_l)
    else:
        tiles = np.zeros(0, np.uint64); ids = np.zeros(0, np.int64); db = np.zeros(0, np.uint64)
    keys = (tiles << np.uint64(32)) | db
    order = np.lexsort((ids, keys))
    keys = keys[order]
    vals = ids[order].astype(np.uint32)
    ranges = np.zeros((T, 2), np.uint32)
    if len(keys):
        t_sorted = (keys >> np.uint64(32)).astype(np.int64)
        bounds = np.searchsorted(t_sorted, np.arange(T + 1))
        cnt = bounds[1:] - bounds[:-1]
        nz = cnt > 0
        ranges[nz, 0] = bounds[:-1][nz]
        ranges[nz, 1] = bounds[1:][nz]
    return keys, vals, ranges


def binning_fast(geom, cam: Camera):
    """Vectorised equivalent of :func:`binning` (used at large sizes)."""
    gx, gy = cam.grid
    T = gx * gy
    vis = np.nonzero(geom["visible"])[0]
    rect = geom["rect"][vis]
    w = rect[:, 2] - rect[:, 0]
    h = rect[:, 3] - rect[:, 1]
    n = w * h
    K = int(n.sum())
    owner = np.repeat(np.arange(len(vis)), n)
    start = np.repeat(np.cumsum(n) - n, n)
    local = np.arange(K) - start
    ww = w[owner]
    ty = rect[owner, 1] + local // np.maximum(ww, 1)
    tx = rect[owner, 0] + local % np.maximum(ww, 1)
    tiles = (ty * gx + tx).astype(np.uint64)
    ids = vis[owner]
    db = geom["depth"][ids].view(np.uint32).astype(np.uint64)
    keys = (tiles << np.uint64(32)) | db
    order = np.lexsort((ids, keys))
    keys = keys[order]
    vals = ids[order].astype(np.uint32)
    ranges = np.zeros((T, 2), np.uint32)
    if K:
        t_sorted = (keys >> np.uint64(32)).astype(np.int64)
        bounds = np.searchsorted(t_sorted, np.arange(T + 1))
        cnt = bounds[1:] - bounds[:-1]
        nz = cnt > 0
        ranges[nz, 0] = bounds[:-1][nz]
        ranges[nz, 1] = bounds[1:][nz]
    return keys, vals, ranges


# ----------------------------------------------------------------------------
# FP64 continuous part
# ----------------------------------------------------------------------------

def eval_sh_rgb(deg, sh, dirs):
    """SH (deg <= 3) -> RGB, the polynomial of ``utils/sh_utils.py:75-99``
    with the reference rasteriser's ``+0.5`` offset.  sh: [P, M, 3]."""
    x, y, z = dirs[:, 0:1], dirs[:, 1:2], dirs[:, 2:3]
    res = SH_C0 * sh[:, 0]
    if deg > 0:
        res = res - SH_C1 * y * sh[:, 1] + SH_C1 * z * sh[:, 2] - SH_C1 * x * sh[:, 3]
        if deg > 1:
            xx, yy, zz = x * x, y * y, z * z
            xy, yz, xz = x * y, y * z, x * z
            res = (res + SH_C2[0] * xy * sh[:, 4] + SH_C2[1] * yz * sh[:, 5]
                   + SH_C2[2] * (2.0 * zz - xx - yy) * sh[:, 6]
                   + SH_C2[3] * xz * sh[:, 7] + SH_C2[4] * (xx - yy) * sh[:, 8])
            if deg > 2:
                res = (res + SH_C3[0] * y * (3 * xx - yy) * sh[:, 9]
                       + SH_C3[1] * xy * z * sh[:, 10]
                       + SH_C3[2] * y * (4 * zz - xx - yy) * sh[:, 11]
                       + SH_C3[3] * z * (2 * zz - 3 * xx - 3 * yy) * sh[:, 12]
                       + SH_C3[4] * x * (4 * zz - xx - yy) * sh[:, 13]
                       + SH_C3[5] * z * (xx - yy) * sh[:, 14]
                       + SH_C3[6] * x * (xx - 3 * yy) * sh[:, 15])
    return res + 0.5


def _quat_to_rot(q):
    r, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = torch.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y),
        2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x),
        2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], 1)
    return R.view(-1, 3, 3)


def _sym_from6(c):
    return torch.stack([c[:, 0], c[:, 1], c[:, 2], c[:, 1], c[:, 3], c[:, 4],
                        c[:, 2], c[:, 4], c[:, 5]], 1).view(-1, 3, 3)


def _straight_min(v, cap):
    """min(v, cap) whose gradient is that of v (the cap is not differentiated)."""
    return v - (v - cap).clamp_min(0).detach()


def project_fp64(cam: Camera, means3D, opacities, shs=None, colors=None,
                 scales=None, rotations=None, cov3D=None, sel=None):
    """Per-Gaussian continuous quantities in FP64 for indices ``sel``.
    Returns ndc [n,2], xy_pix [n,2], conic [n,3], opac [n], rgb [n,3]."""
    m = means3D[sel]
    V = torch.as_tensor(np.asarray(cam.viewmatrix, np.float64).reshape(4, 4))
    Pm = torch.as_tensor(np.asarray(cam.projmatrix, np.float64).reshape(4, 4))
    ones = torch.ones(m.shape[0], 1, dtype=m.dtype)
    mh = torch.cat([m, ones], 1)
    view = mh @ V          # row-vector convention: [x y z 1] @ V
    hom = mh @ Pm
    pw = 1.0 / (hom[:, 3:4] + 1e-7)
    ndc = hom[:, :2] * pw
    W, H = float(cam.width), float(cam.height)
    pix = torch.stack([((ndc[:, 0] + 1) * W - 1) * 0.5, ((ndc[:, 1] + 1) * H - 1) * 0.5], 1)

    if cov3D is None:
        s = scales[sel] * cam.scale_modifier
        R = _quat_to_rot(rotations[sel])
        M = R * s[:, None, :]
        Sig = M @ M.transpose(1, 2)
    else:
        Sig = _sym_from6(cov3D[sel])

    fx = W / (2.0 * cam.tanfovx)
    fy = H / (2.0 * cam.tanfovy)
    vx, vy, vz = view[:, 0], view[:, 1], view[:, 2]
    limx, limy = 1.3 * cam.tanfovx, 1.3 * cam.tanfovy
    with torch.no_grad():
        rx = vx / vz
        ry = vy / vz
        clx = (rx < -limx) | (rx > limx)
        cly = (ry < -limy) | (ry > limy)
        tx_c = rx.clamp(-limx, limx) * vz
        ty_c = ry.clamp(-limy, limy) * vz
    tx = torch.where(clx, tx_c, vx)
    ty = torch.where(cly, ty_c, vy)
    zero = torch.zeros_like(vz)
    J = torch.stack([fx / vz, zero, -fx * tx / (vz * vz),
                     zero, fy / vz, -fy * ty / (vz * vz)], 1).view(-1, 2, 3)
    Wr = V[:3, :3].T  # world->view rotation (math convention)
    Tm = J @ Wr
    c2 = Tm @ Sig @ Tm.transpose(1, 2)
    a = c2[:, 0, 0] + 0.3
    b = c2[:, 0, 1]
    c = c2[:, 1, 1] + 0.3
    det = a * c - b * b
    conic = torch.stack([c / det, -b / det, a / det], 1)

    if colors is None:
        campos = torch.as_tensor(np.asarray(cam.campos, np.float64).reshape(1, 3))
        d = m - campos
        d = d / d.norm(dim=1, keepdim=True)
        rgb = eval_sh_rgb(cam.sh_degree, shs[sel], d).clamp_min(0.0)
    else:
        rgb = colors[sel]
    op = opacities[sel].reshape(-1)
    return ndc, pix, conic, op, rgb


def _blend_tile(pix_xy, xy, conic, op, rgb, bg):
    """Front-to-back blending of one tile.  pix_xy [n_pix,2] float64 pixel
    coordinates; xy/conic/op/rgb: the tile's Gaussians in depth order."""
    d = xy.unsqueeze(0) - pix_xy.unsqueeze(1)               # [npix, n, 2]
    co = conic.unsqueeze(0)
    power = -0.5 * (co[..., 0] * d[..., 0] ** 2 + co[..., 2] * d[..., 1] ** 2) - co[..., 1] * d[..., 0] * d[..., 1]
    G = torch.exp(power)
    araw = op.unsqueeze(0) * G
    alpha = _straight_min(araw, 0.99)
    with torch.no_grad():
        valid = (power <= 0) & (alpha >= 1.0 / 255.0)
        a_v = torch.where(valid, alpha, torch.zeros_like(alpha))
        T_after = torch.cumprod(1 - a_v, dim=1)
        keep = T_after >= 1e-4
        # ambiguity: a decision within FP32 reach of its threshold, before
        # termination.  An FP32 kernel holds the projected mean to about an
        # ulp of its pixel coordinates (a few roundings: 4 ulp), which moves
        # the exponent by |d power / d mean| times that, and evaluates the
        # exponent's terms to a few ulp: the alpha test's relative band is
        # the larger of 1e-5 and that reach; the transmittance test's band
        # adds up the bands of the alphas blended before it.
        processed = torch.cat([torch.ones_like(keep[:, :1]), keep[:, :-1]], 1)
        ulp = lambda v: torch.ldexp(torch.ones_like(v), torch.frexp(v.abs().clamp_min(1.0))[1] - 24)  # noqa: E731
        gx = (co[..., 0] * d[..., 0] + co[..., 1] * d[..., 1]).abs()
        gy = (co[..., 2] * d[..., 1] + co[..., 1] * d[..., 0]).abs()
        terms = (0.5 * co[..., 0] * d[..., 0] ** 2).abs() + (0.5 * co[..., 2] * d[..., 1] ** 2).abs() + \
            (co[..., 1] * d[..., 0] * d[..., 1]).abs()
        reach = 4.0 * (gx * ulp(xy[:, 0]).unsqueeze(0) + gy * ulp(xy[:, 1]).unsqueeze(0)) + \
            4.0 * 2.0 ** -23 * terms
        band_a = torch.clamp_min(reach, 1e-5)
        amb_a = ((alpha - 1.0 / 255.0).abs() <= band_a / 255.0) & (power <= 0)
        band_t = 1e-5 + torch.cumsum(a_v * band_a / (1 - a_v), dim=1)
        amb_t = valid & ((T_after - 1e-4).abs() <= band_t * 1e-4)
        ambiguous = ((amb_a | amb_t) & processed).any(1)
        use = valid & keep
        idx = torch.arange(1, use.shape[1] + 1).unsqueeze(0).expand_as(use)
        n_contrib = torch.where(use, idx, torch.zeros_like(idx)).max(1).values
    a_k = torch.where(use, alpha, torch.zeros_like(alpha))
    one_minus = 1 - a_k
    T_incl = torch.cumprod(one_minus, dim=1)
    T_before = torch.cat([torch.ones_like(T_incl[:, :1]), T_incl[:, :-1]], 1)
    w = a_k * T_before
    C = w @ rgb                                               # [npix, 3]
    T_final = T_incl[:, -1]
    out = C + T_final.unsqueeze(1) * bg.view(1, 3)
    return out, T_final, n_contrib, ambiguous


class OracleResult:
    """Forward outputs of :func:`render` plus a ``backward(dL_dimage)``."""


def render(cam: Camera, means3D, opacities, shs=None, colors=None, scales=None,
           rotations=None, cov3D=None, tiles_subset=None, want_backward=True):
    """Full oracle forward.  Array inputs are numpy float32 (the kernel's
    inputs); the FP64 part promotes them.  ``tiles_subset``: optional list of
    tile ids to blend (others are left as background) — used to bound the
    CPU-time of the baseline sample.

    Returns an object with image [3,H,W] f64, radii, final_T, n_contrib,
    ambiguous [H,W], binning outputs, and ``backward(dL_dimage)`` returning a
    dict of gradients (numpy float64) with the reference's output names.
    """
    geom = geometry_f32(means3D, cam, opacities, scales, rotations, cov3D)
    keys, vals, ranges = binning_fast(geom, cam)
    P = means3D.shape[0]
    W, H = cam.width, cam.height
    gx, gy = cam.grid
    vis = np.nonzero(geom["visible"])[0]
    sel = torch.as_tensor(vis, dtype=torch.long)
    leaves = {}
    def leaf(name, arr):
        if arr is None:
            return None
        t = torch.as_tensor(np.asarray(arr, np.float64)).clone().requires_grad_(want_backward)
        leaves[name] = t
        return t
    t_means = leaf("means3D", means3D)
    t_op = leaf("opacities", np.asarray(opacities).reshape(P, 1))
    t_shs = leaf("shs", shs)
    t_col = leaf("colors_precomp", colors)
    t_sc = leaf("scales", scales)
    t_rot = leaf("rotations", rotations)
    t_cov = leaf("cov3D_precomp", cov3D)
    ndc, pix, conic, op, rgb = project_fp64(cam, t_means, t_op, t_shs, t_col, t_sc, t_rot, t_cov, sel)
    # detached per-Gaussian leaves for the (memory-bounded) per-tile blend
    ndc_l = ndc.detach().clone().requires_grad_(want_backward)
    conic_l = conic.detach().clone().requires_grad_(want_backward)
    op_l = op.detach().clone().requires_grad_(want_backward)
    rgb_l = rgb.detach().clone().requires_grad_(want_backward)
    remap = np.full(P, -1, np.int64)
    remap[vis] = np.arange(len(vis))
    bg = torch.as_tensor(np.asarray(cam.bg, np.float64).reshape(3))

    def pix_of_ndc(n):
        return torch.stack([((n[:, 0] + 1) * W - 1) * 0.5, ((n[:, 1] + 1) * H - 1) * 0.5], 1)

    image = bg.view(3, 1, 1).expand(3, H, W).clone()
    final_T = torch.ones(H, W, dtype=torch.float64)
    n_contrib = torch.zeros(H, W, dtype=torch.int64)
    ambiguous = torch.zeros(H, W, dtype=torch.bool)
    tiles = range(gx * gy) if tiles_subset is None else tiles_subset
    with torch.no_grad():
        xy_all = pix_of_ndc(ndc_l)
    tile_info = []
    for t in tiles:
        ty, tx = divmod(int(t), gx)
        x0, y0 = tx * BLOCK, ty * BLOCK
        x1, y1 = min(x0 + BLOCK, W), min(y0 + BLOCK, H)
        yy, xx = torch.meshgrid(torch.arange(y0, y1, dtype=torch.float64),
                                torch.arange(x0, x1, dtype=torch.float64), indexing="ij")
        pxy = torch.stack([xx.reshape(-1), yy.reshape(-1)], 1)
        r0, r1 = ranges[t]
        g = torch.as_tensor(remap[vals[r0:r1].astype(np.int64)])
        if len(g) == 0:
            continue
        with torch.no_grad():
            out, Tf, nc, amb = _blend_tile(pxy, xy_all[g], conic_l[g], op_l[g], rgb_l[g], bg)
        image[:, y0:y1, x0:x1] = out.T.reshape(3, y1 - y0, x1 - x0)
        final_T[y0:y1, x0:x1] = Tf.reshape(y1 - y0, x1 - x0)
        n_contrib[y0:y1, x0:x1] = nc.reshape(y1 - y0, x1 - x0)
        ambiguous[y0:y1, x0:x1] = amb.reshape(y1 - y0, x1 - x0)
        tile_info.append((t, x0, y0, x1, y1, pxy, g))

    res = OracleResult()
    res.image = image.numpy()
    res.final_T = final_T.numpy()
    res.n_contrib = n_contrib.numpy()
    res.ambiguous = ambiguous.numpy()
    res.geom = geom
    res.keys, res.values, res.ranges = keys, vals, ranges
    res.radii = geom["radii"]
    res.num_rendered = int(len(keys))

    def backward(dL_dimage):
        gimg = torch.as_tensor(np.asarray(dL_dimage, np.float64))
        for (t, x0, y0, x1, y1, pxy, g) in tile_info:
            out, _, _, _ = _blend_tile(pxy, pix_of_ndc(ndc_l[g]), conic_l[g], op_l[g], rgb_l[g], bg)
            go = gimg[:, y0:y1, x0:x1].reshape(3, -1).T
            torch.autograd.backward(out, go)
        grads_2d = [x.grad if x.grad is not None else torch.zeros_like(x) for x in (ndc_l, conic_l, op_l, rgb_l)]
        torch.autograd.backward([ndc, conic, op, rgb], grads_2d)
        out = {}
        for name, t in leaves.items():
            out[name] = (t.grad if t.grad is not None else torch.zeros_like(t)).numpy()
        gm2 = np.zeros((P, 3))
        gm2[vis, :2] = grads_2d[0].numpy()
        out["means2D"] = gm2
        return out

    res.backward = backward
    return res


def mark_visible(means3D, viewmatrix):
    """Frustum test of ``markVisible``: visible iff view-space z > 0.2."""
    m = means3D.astype(F32)
    V = np.asarray(viewmatrix, F32).reshape(16)
    vz = ((V[2] * m[:, 0] + V[6] * m[:, 1]) + V[10] * m[:, 2]) + V[14]
    return vz > F32(0.2)
