"""The renderer's Python-side colour path in one kernel (csrc/shcolor.cu).

``sh_colors(deg, sh, xyz, campos)`` equals
``torch.sigmoid(eval_sh(deg, sh, normalize(xyz - campos)))`` — the
``convert_SHs_python`` branch of ``render`` / ``render_dyn``
(gaussian_renderer/__init__.py:70-78, :162-170) — for ``sh`` [P, 3, K]
(channel-major, as ``features.view(-1, 3, K)`` there), differentiable w.r.t.
``sh`` and ``xyz`` (the camera centre is a constant there too).
"""
from __future__ import annotations

import torch

from . import _lib
from ._lib import check, stream_of

__all__ = ["sh_colors"]


class _SHColors(torch.autograd.Function):
    @staticmethod
    def forward(ctx, deg, sh, xyz, campos):
        lib = _lib.load()
        s = sh.detach().float().contiguous()
        x = xyz.detach().float().contiguous()
        c = campos.detach().float().contiguous().to(x.device)
        P, K = s.shape[0], s.shape[2]
        out = torch.empty((P, 3), dtype=torch.float32, device=x.device)
        check(lib.dmgs_sh_colors_fwd(P, int(deg), K, s.data_ptr(), x.data_ptr(), c.data_ptr(),
                                     out.data_ptr(), stream_of(x.device)), "sh_colors_fwd")
        ctx.deg = int(deg)
        ctx.save_for_backward(s, x, c)
        return out

    @staticmethod
    def backward(ctx, dcolors):
        lib = _lib.load()
        s, x, c = ctx.saved_tensors
        g = dcolors.float().contiguous()
        dsh = torch.empty_like(s)
        dx = torch.empty_like(x) if ctx.needs_input_grad[2] else None
        check(lib.dmgs_sh_colors_bwd(s.shape[0], ctx.deg, s.shape[2], s.data_ptr(), x.data_ptr(),
                                     c.data_ptr(), g.data_ptr(), dsh.data_ptr(),
                                     None if dx is None else dx.data_ptr(), stream_of(x.device)),
              "sh_colors_bwd")
        return None, dsh, dx, None


def sh_colors(deg, sh, xyz, campos):
    """sigmoid(SH_deg(dir)) per Gaussian: sh [P, 3, K], xyz [P, 3], campos
    [3] -> colours [P, 3]."""
    if not xyz.is_cuda:
        raise RuntimeError("sh_colors: inputs must be CUDA tensors (no CPU path)")
    if sh.dim() != 3 or sh.shape[1] != 3 or sh.shape[0] != xyz.shape[0]:
        raise ValueError("sh_colors: sh must be [P, 3, K] with P = xyz.shape[0]")
    if not 0 <= int(deg) <= 3 or sh.shape[2] < (int(deg) + 1) ** 2:
        raise ValueError("sh_colors: degree 0..3 with K >= (deg + 1)^2")
    return _SHColors.apply(int(deg), sh, xyz, campos)
