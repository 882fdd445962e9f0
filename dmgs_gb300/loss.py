"""Fused photometric loss: (1 - lambda) L1 + lambda (1 - SSIM) and its
gradient in two kernels (csrc/loss.cu), in place of the reference's torch
composition (utils/loss_utils.py, train_geo_stage2.py:114-116)."""
from __future__ import annotations

import torch

from . import _lib
from ._lib import check, stream_of


class _L1SSIM(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image, target, lambda_dssim):
        lib = _lib.load()
        x = image.detach().float().contiguous()
        y = target.detach().float().contiguous()
        C, H, W = x.shape
        scratch = torch.empty(lib.dmgs_l1_ssim_scratch_bytes(C, H, W), dtype=torch.uint8,
                              device=x.device)
        loss = torch.empty((), device=x.device)
        grad = torch.empty_like(x)
        check(lib.dmgs_l1_ssim(x.data_ptr(), y.data_ptr(), C, H, W, float(lambda_dssim),
                               loss.data_ptr(), grad.data_ptr(), scratch.data_ptr(),
                               scratch.numel(), stream_of(x.device)), "l1_ssim")
        ctx.save_for_backward(grad)
        return loss

    @staticmethod
    def backward(ctx, dloss):
        (grad,) = ctx.saved_tensors
        return grad * dloss, None, None


def l1_ssim_loss(image, target, lambda_dssim=0.2):
    """(1 - lambda) mean|image - target| + lambda (1 - mean SSIM) for [C,H,W]
    images; differentiable w.r.t. image."""
    return _L1SSIM.apply(image, target, lambda_dssim)
