"""Drop-in ``diff_gaussian_rasterization`` surface backed by libdmgs_gb300.so.

Same names, fields, argument meaning and errors as the module the reference
imports at ``gaussian_renderer/__init__.py:14`` and calls at :36-51, :86-94
(``render``) and :129-144, :178-186 (``render_dyn``):

* ``GaussianRasterizationSettings`` — 12-field NamedTuple;
* ``GaussianRasterizer(raster_settings)`` — ``nn.Module`` whose
  ``forward(means3D, means2D, opacities, shs=None, colors_precomp=None,
  scales=None, rotations=None, cov3D_precomp=None)`` returns
  ``(color [3,H,W], radii [P] int32)`` and ``markVisible(positions)``;
* ``rasterize_gaussians(...)`` — the autograd entry.

The gradient written into ``means2D.grad`` is w.r.t. NDC (x, y) — the
screen-space quantity the reference's densification reads
(``scene/gaussian_model.py:405-406``).

Everything runs on the caller's current CUDA stream.  The forward pass
synchronises once (to size the tile-instance buffers), like the reference.
"""
from __future__ import annotations

import math
from typing import NamedTuple

import torch
import torch.nn as nn

from . import _lib
from ._lib import DmgsGaussians, DmgsGrads, DmgsView, check, ptr, stream_of


class GaussianRasterizationSettings(NamedTuple):
    image_height: int
    image_width: int
    tanfovx: float
    tanfovy: float
    bg: torch.Tensor
    scale_modifier: float
    viewmatrix: torch.Tensor
    projmatrix: torch.Tensor
    sh_degree: int
    campos: torch.Tensor
    prefiltered: bool
    debug: bool


def _f32(t, device):
    if t is None:
        return None
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(t)
    if t.numel() == 0:
        return None
    t = t.to(device=device, dtype=torch.float32)
    if not t.is_contiguous():
        t = t.contiguous()
    return t


def _dims(t):
    return tuple(t.shape) if hasattr(t, "shape") else tuple(torch.as_tensor(t).shape)


def check_inputs(means3D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None,
                 cov3D_precomp=None, settings=()):
    """Shapes of the arrays the kernels index, checked on the host before any
    device work (the reference's extension rejects a means3D that is not
    [P, 3] with the same message).  Empty arrays count as absent, as in the
    reference's wrapper; which inputs must be present is the input-mode rule,
    checked separately."""
    if means3D is None or len(_dims(means3D)) != 2 or _dims(means3D)[1] != 3:
        raise RuntimeError("means3D must have dimensions (num_points, 3)")
    P = _dims(means3D)[0]
    present = lambda t: t is not None and math.prod(_dims(t)) > 0  # noqa: E731
    if opacities is None or math.prod(_dims(opacities)) != P:
        got = None if opacities is None else list(_dims(opacities))
        raise RuntimeError(f"opacities must hold one value per point ({P}), got {got}")
    if present(shs):
        d = _dims(shs)
        if len(d) != 3 or d[0] != P or d[2] != 3:
            raise RuntimeError(f"shs must have dimensions (num_points, M, 3), got {list(d)}")
    for name, t, w in (("colors_precomp", colors_precomp, 3), ("scales", scales, 3),
                       ("rotations", rotations, 4), ("cov3D_precomp", cov3D_precomp, 6)):
        if present(t) and _dims(t) != (P, w):
            raise RuntimeError(f"{name} must have dimensions (num_points, {w}), got {list(_dims(t))}")
    for rs in settings:
        for name, n in (("bg", 3), ("viewmatrix", 16), ("projmatrix", 16), ("campos", 3)):
            t = getattr(rs, name)
            if t is None or math.prod(_dims(t)) != n:
                raise RuntimeError(f"raster settings: {name} must hold {n} values")


def _aligned16(t):
    if t is not None and t.data_ptr() % 16 != 0:
        t = t.clone()
    return t


def make_view(rs: GaussianRasterizationSettings, device, keep):
    """Fill a DmgsView; `keep` collects the tensors whose addresses it holds."""
    bg = _f32(rs.bg, device)
    vm = _f32(rs.viewmatrix, device)
    pm = _f32(rs.projmatrix, device)
    cp = _f32(rs.campos, device)
    keep.extend([bg, vm, pm, cp])
    return DmgsView(int(rs.image_width), int(rs.image_height), float(rs.tanfovx),
                    float(rs.tanfovy), float(rs.scale_modifier), int(rs.sh_degree),
                    int(bool(rs.prefiltered)), int(bool(rs.debug)),
                    ptr(bg), ptr(vm), ptr(pm), ptr(cp))


def _snapshot(name, args):
    try:
        torch.save([a.detach().cpu() if isinstance(a, torch.Tensor) else a for a in args], name)
        print(f"\nAn error occured in the rasteriser. Writing snapshot to {name} for debugging.")
    except Exception:  # pragma: no cover - best effort, as in the reference wrapper
        pass


class _RasterizeGaussians(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means3D, means2D, sh, colors_precomp, opacities, scales, rotations,
                cov3Ds_precomp, raster_settings):
        check_inputs(means3D, opacities, sh, colors_precomp, scales, rotations, cov3Ds_precomp,
                     (raster_settings,))
        lib = _lib.load()
        device = means3D.device
        if device.type != "cuda":
            raise RuntimeError("the GB300 rasteriser needs CUDA tensors (no CPU fallback)")
        means3D = _f32(means3D, device)
        opac = _f32(opacities, device)
        sh = _f32(sh, device)
        colors = _f32(colors_precomp, device)
        scales = _f32(scales, device)
        rotations = _aligned16(_f32(rotations, device))
        cov3D = _f32(cov3Ds_precomp, device)
        P = means3D.shape[0]
        M = sh.shape[1] if sh is not None else 0
        H, W = int(raster_settings.image_height), int(raster_settings.image_width)
        keep = []
        view = make_view(raster_settings, device, keep)
        g = DmgsGaussians(P, M, ptr(means3D), ptr(opac), ptr(sh), ptr(colors), ptr(scales),
                          ptr(rotations), ptr(cov3D))
        stream = stream_of(device)
        geom = torch.empty(lib.dmgs_geom_state_bytes(P, W, H), dtype=torch.uint8, device=device)
        radii = torch.empty(P, dtype=torch.int32, device=device)
        K = _lib.C.c_int64(0)
        try:
            check(lib.dmgs_raster_fwd_geometry(view, g, geom.data_ptr(), geom.numel(),
                                               ptr(radii), _lib.C.byref(K), stream),
                  "rasterize_gaussians")
            K = int(K.value)
            binning = torch.empty(lib.dmgs_binning_state_bytes(K, W, H), dtype=torch.uint8,
                                  device=device)
            img = torch.empty(lib.dmgs_image_state_bytes(W, H), dtype=torch.uint8, device=device)
            color = torch.empty(3, H, W, dtype=torch.float32, device=device)
            check(lib.dmgs_raster_fwd_render(view, g, geom.data_ptr(), geom.numel(),
                                             binning.data_ptr(), binning.numel(), K,
                                             img.data_ptr(), img.numel(), color.data_ptr(), stream),
                  "rasterize_gaussians")
        except Exception:
            if raster_settings.debug:
                _snapshot("snapshot_fw.dump", [means3D, colors, opac, scales, rotations, cov3D, sh,
                                               raster_settings.viewmatrix, raster_settings.projmatrix,
                                               raster_settings.campos])
            raise
        ctx.raster_settings = raster_settings
        ctx.num_rendered = K
        ctx.M = M
        ctx.opac_shape = tuple(opacities.shape)
        ctx.save_for_backward(means3D, colors, opac, scales, rotations, cov3D, radii, sh,
                              geom, binning, img)
        ctx.mark_non_differentiable(radii)
        return color, radii

    @staticmethod
    def backward(ctx, grad_out_color, _grad_radii):
        lib = _lib.load()
        rs = ctx.raster_settings
        (means3D, colors, opac, scales, rotations, cov3D, radii, sh, geom, binning,
         img) = ctx.saved_tensors
        device = means3D.device
        P = means3D.shape[0]
        M = ctx.M
        H, W = int(rs.image_height), int(rs.image_width)
        keep = []
        view = make_view(rs, device, keep)
        g = DmgsGaussians(P, M, ptr(means3D), ptr(opac), ptr(sh), ptr(colors), ptr(scales),
                          ptr(rotations), ptr(cov3D))
        dout = _f32(grad_out_color, device)
        z = lambda *s: torch.empty(*s, dtype=torch.float32, device=device)  # noqa: E731
        d_means2D = z(P, 3)
        d_colors = z(P, 3)
        d_opac = z(P, 1)
        d_means3D = z(P, 3)
        d_cov3D = z(P, 6) if cov3D is not None else None
        d_sh = z(P, M, 3) if sh is not None else None
        d_scales = z(P, 3) if scales is not None and cov3D is None else None
        d_rot = z(P, 4) if rotations is not None and cov3D is None else None
        grads = DmgsGrads(ptr(d_means2D), ptr(d_colors), ptr(d_opac), ptr(d_means3D),
                          ptr(d_cov3D), ptr(d_sh), ptr(d_scales), ptr(d_rot))
        scratch = torch.empty(lib.dmgs_bwd_scratch_bytes(P), dtype=torch.uint8, device=device)
        try:
            check(lib.dmgs_raster_bwd(view, g, ptr(dout), geom.data_ptr(), geom.numel(),
                                      binning.data_ptr(), binning.numel(), ctx.num_rendered,
                                      img.data_ptr(), img.numel(), scratch.data_ptr(),
                                      scratch.numel(), grads, stream_of(device)),
                  "rasterize_gaussians_backward")
        except Exception:
            if rs.debug:
                _snapshot("snapshot_bw.dump", [means3D, radii, colors, scales, rotations, cov3D, dout,
                                               sh, rs.viewmatrix, rs.projmatrix, rs.campos])
            raise
        return (d_means3D, d_means2D, d_sh, d_colors if colors is not None else None,
                d_opac.view(ctx.opac_shape), d_scales, d_rot, d_cov3D, None)


def rasterize_gaussians(means3D, means2D, sh, colors_precomp, opacities, scales, rotations,
                        cov3Ds_precomp, raster_settings):
    return _RasterizeGaussians.apply(means3D, means2D, sh, colors_precomp, opacities, scales,
                                     rotations, cov3Ds_precomp, raster_settings)


class GaussianRasterizer(nn.Module):
    def __init__(self, raster_settings):
        super().__init__()
        self.raster_settings = raster_settings

    def markVisible(self, positions):
        """Frustum test: True where view-space z > 0.2."""
        lib = _lib.load()
        rs = self.raster_settings
        with torch.no_grad():
            pos = _f32(positions, positions.device)
            vm = _f32(rs.viewmatrix, positions.device)
            pm = _f32(rs.projmatrix, positions.device)
            out = torch.empty(pos.shape[0], dtype=torch.uint8, device=positions.device)
            check(lib.dmgs_mark_visible(pos.shape[0], ptr(pos), ptr(vm), ptr(pm), ptr(out),
                                        stream_of(positions.device)), "mark_visible")
        return out.bool()

    def forward(self, means3D, means2D, opacities, shs=None, colors_precomp=None, scales=None,
                rotations=None, cov3D_precomp=None):
        rs = self.raster_settings
        if (shs is None and colors_precomp is None) or (shs is not None and colors_precomp is not None):
            raise Exception('Please provide exactly one of either SHs or precomputed colors!')
        if ((scales is None or rotations is None) and cov3D_precomp is None) or \
                ((scales is not None or rotations is not None) and cov3D_precomp is not None):
            raise Exception('Please provide exactly one of either scale/rotation pair or precomputed 3D covariance!')
        return rasterize_gaussians(means3D, means2D, shs, colors_precomp, opacities, scales,
                                   rotations, cov3D_precomp, rs)
