"""Hash-grid texture on the GPU (csrc/texture.cu): the drop-in for the
reference's ``geo.texture.MLPTexture3D`` (geo/texture.py:47-118), whose
encoding is tiny-cuda-nn's HashGrid and whose MLP is a bias-free ReLU net
(32 -> 32 -> 32 -> channels).

Same constructor, ``sample`` / ``sample_noact``, parameters and
``state_dict`` keys (``encoder.params``, ``net.net.0.weight``,
``net.net.2.weight``, ``net.net.4.weight``), so a reference checkpoint loads
as is.  ``sample_noact`` runs the encoding and the MLP in one kernel and
its adjoint in another; the gradient reaching ``encoder.params`` is 128x the
true one and the gradient w.r.t. the positions is the true one, as the
reference's hooks (geo/texture.py:72-73, ``_MLP``'s loss_scale) leave them.
The encoding runs in float32 (tiny-cuda-nn's default is half precision).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, stream_of

__all__ = ["MLPTexture3D"]

N_LEVELS, N_FEATURES, LOG2_HASHMAP, BASE_RES, DESIRED_RES = 16, 2, 19, 16, 4096
GRADIENT_SCALING = 128.0


def _desc(aabb, table, W1, W2, W3, channels, per_level_scale):
    d = _lib.DmgsTexture()
    d.table, d.W1, d.W2, d.W3 = table.data_ptr(), W1.data_ptr(), W2.data_ptr(), W3.data_ptr()
    d.channels = channels
    lo_hi = [float(v) for v in aabb.reshape(-1).tolist()]
    d.aabb = (C.c_float * 6)(*lo_hi)
    d.per_level_scale = per_level_scale
    return d


class _TextureFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, table, W1, W2, W3, aabb_host, per_level_scale, keep_enc):
        lib = _lib.load()
        x = xyz.detach().float().contiguous()
        t, w1, w2, w3 = (a.detach().float().contiguous() for a in (table, W1, W2, W3))
        channels = w3.shape[0]
        d = _desc(aabb_host, t, w1, w2, w3, channels, per_level_scale)
        out = torch.empty((x.shape[0], channels), dtype=torch.float32, device=x.device)
        if keep_enc:
            # keep the encoding for the adjoint (128 B per point) instead of
            # recomputing its table gathers there
            enc = torch.empty((x.shape[0], 32), dtype=torch.float32, device=x.device)
            check(lib.dmgs_tex_fwd_enc(C.byref(d), x.shape[0], ptr(x), ptr(out), ptr(enc),
                                       stream_of(x.device)), "tex_fwd")
        else:
            enc = None
            check(lib.dmgs_tex_fwd(C.byref(d), x.shape[0], ptr(x), ptr(out), stream_of(x.device)),
                  "tex_fwd")
        ctx.save_for_backward(x, t, w1, w2, w3, enc)
        ctx.aabb, ctx.pls = aabb_host, per_level_scale
        return out

    @staticmethod
    def backward(ctx, dout):
        lib = _lib.load()
        x, t, w1, w2, w3, enc = ctx.saved_tensors
        d = _desc(ctx.aabb, t, w1, w2, w3, w3.shape[0], ctx.pls)
        g = dout.float().contiguous()
        dx = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        dt = torch.empty_like(t) if ctx.needs_input_grad[1] else None
        dw1, dw2, dw3 = torch.empty_like(w1), torch.empty_like(w2), torch.empty_like(w3)
        scratch = torch.empty(max(1, lib.dmgs_tex_bwd_scratch_bytes(x.shape[0]) // 4),
                              dtype=torch.float32, device=x.device)
        if enc is not None:
            check(lib.dmgs_tex_bwd_enc(C.byref(d), x.shape[0], ptr(x), ptr(enc), ptr(g), ptr(dx),
                                       ptr(dt), dw1.data_ptr(), dw2.data_ptr(), dw3.data_ptr(),
                                       scratch.data_ptr(), scratch.numel() * 4,
                                       stream_of(x.device)), "tex_bwd")
        else:
            check(lib.dmgs_tex_bwd(C.byref(d), x.shape[0], ptr(x), ptr(g), ptr(dx), ptr(dt),
                                   dw1.data_ptr(), dw2.data_ptr(), dw3.data_ptr(), scratch.data_ptr(),
                                   scratch.numel() * 4, stream_of(x.device)), "tex_bwd")
        return dx, dt, dw1, dw2, dw3, None, None, None


class _HashGridParams(torch.nn.Module):
    """Holds the encoding's table as ``params`` (the name the reference's
    state dict uses), initialised uniformly in [-1e-4, 1e-4]."""

    def __init__(self, entries, device):
        super().__init__()
        self.params = torch.nn.Parameter(
            (torch.rand(entries * N_FEATURES, device=device) * 2 - 1) * 1e-4)
        self.n_output_dims = N_LEVELS * N_FEATURES


class _MLP(torch.nn.Module):
    """Bias-free ReLU MLP with the reference's layout and initialisation
    (geo/texture.py:18-40); its forward is the fused kernel's."""

    def __init__(self, n_in, n_neurons, n_hidden, n_out, device):
        super().__init__()
        layers = [torch.nn.Linear(n_in, n_neurons, bias=False), torch.nn.ReLU()]
        for _ in range(n_hidden - 1):
            layers += [torch.nn.Linear(n_neurons, n_neurons, bias=False), torch.nn.ReLU()]
        layers += [torch.nn.Linear(n_neurons, n_out, bias=False)]
        self.net = torch.nn.Sequential(*layers).to(device)
        for m in self.net:
            if isinstance(m, torch.nn.Linear):
                torch.nn.init.kaiming_uniform_(m.weight, nonlinearity="relu")

    def weights(self):
        return [m.weight for m in self.net if isinstance(m, torch.nn.Linear)]


class MLPTexture3D(torch.nn.Module):
    def __init__(self, AABB, channels=3, internal_dims=32, hidden=2, min_max=None, device="cuda"):
        super().__init__()
        if internal_dims != 32 or hidden != 2:
            raise NotImplementedError("MLPTexture3D: the kernels implement 32 neurons x 2 hidden layers "
                                      "(the reference's configuration)")
        if channels not in (3, 12, 27, 48):
            raise NotImplementedError("MLPTexture3D: channels must be 3 (deg + 1)^2 for SH degree <= 3")
        self.channels = channels
        self.internal_dims = internal_dims
        self.AABB = AABB
        self.min_max = min_max
        self.per_level_scale = float(np.exp(np.log(DESIRED_RES / BASE_RES) / (N_LEVELS - 1)))
        entries = int(_lib.load().dmgs_tex_table_entries(C.c_float(self.per_level_scale)))
        self.encoder = _HashGridParams(entries, device)
        self.net = _MLP(N_LEVELS * N_FEATURES, internal_dims, hidden, channels, device)

    def _aabb_host(self):
        """The AABB as a host float32 [2, 3] tensor for the kernel arguments,
        copied again only when ``self.AABB`` is replaced or modified in place
        (a device AABB would otherwise cost a device->host sync per call)."""
        a = self.AABB
        version = getattr(a, "_version", None)
        if getattr(self, "_aabb_src", None) is not a or self._aabb_ver != version:
            self._aabb_cache = torch.as_tensor(a, dtype=torch.float32).detach().cpu().reshape(2, 3).clone()
            self._aabb_src, self._aabb_ver = a, version
        return self._aabb_cache

    def sample_noact(self, texc):
        """Features [..., channels] at positions texc [..., 3]
        (geo/texture.py:101-112)."""
        if texc.numel() == 0:
            return torch.zeros(*texc.shape[:-1], self.channels, device=texc.device)
        W1, W2, W3 = self.net.weights()
        keep = torch.is_grad_enabled() and any(
            t.requires_grad for t in (texc, self.encoder.params, W1, W2, W3))
        out = _TextureFn.apply(texc.reshape(-1, 3), self.encoder.params, W1, W2, W3,
                               self._aabb_host(), self.per_level_scale, keep)
        return out.view(*texc.shape[:-1], self.channels)

    def sample(self, texc):
        """sigmoid(features) scaled into [min_max[0], min_max[1]]
        (geo/texture.py:87-99)."""
        out = torch.sigmoid(self.sample_noact(texc).reshape(-1, self.channels))
        out = out * (self.min_max[1][None, :] - self.min_max[0][None, :]) + self.min_max[0][None, :]
        return out.view(*texc.shape[:-1], self.channels)

    def clamp_(self):
        pass

    def cleanup(self):
        pass
