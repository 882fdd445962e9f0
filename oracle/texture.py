"""Hash-grid texture (positions -> SH features) — CPU oracle, TEST
INFRASTRUCTURE ONLY.

The reference's ``MLPTexture3D`` (``geo/texture.py:47-118``) encodes a
position with tiny-cuda-nn's multiresolution ``HashGrid`` (16 levels x 2
features, 2^19 entries per level, base resolution 16, finest 4096) and maps
the 32 features through a bias-free ReLU MLP (32 -> 32 -> 32 -> channels,
``_MLP``, ``geo/texture.py:18-40``).  Stage 2 calls ``sample_noact`` on the
Gaussians' positions to get their SH coefficients
(``scene/gaussian_geo_model_mlp_flex.py:313``).

Parity:
* The encoding lives in the third-party package tiny-cuda-nn
  (NVlabs/tiny-cuda-nn, installed from the git head without networks,
  ``README.md:15``; no version pinned), absent here.  ``encode`` restates the
  published algorithm (Mueller et al., "Instant Neural Graphics Primitives
  with a Multiresolution Hash Encoding", 2022) with tiny-cuda-nn's documented
  grid conventions: per-level scale 2^(l log2 b) N_min - 1, resolution
  ceil(scale) + 1, position p s + 1/2 split into integer cell and fraction,
  dense indexing (x fastest) while the level's grid fits its table, else the
  spatial hash XOR_d p_d pi_d with pi = (1, 2654435761, 805459861), index
  modulo the level's table size (rounded up to 8), trilinear weights.  It
  runs in float64 here; tiny-cuda-nn's default runs the encoding in half
  precision.  ENCODING PARITY UNPINNED.
* Everything around it — the AABB normalisation and clamp, the MLP's layer
  structure, the output layout and the two gradient-scaling hooks — is
  pinned to the reference's own ``MLPTexture3D`` run on the CPU with this
  encoding in place of tiny-cuda-nn (``tests/golden/make_texture_golden.py``).
"""
from __future__ import annotations

import math

import numpy as np
import torch

N_LEVELS = 16
N_FEATURES = 2
LOG2_HASHMAP = 19
BASE_RES = 16
DESIRED_RES = 4096
PRIMES = (1, 2654435761, 805459861)
GRADIENT_SCALING = 128.0  # geo/texture.py:72-73


def per_level_scale():
    """geo/texture.py:57-60"""
    return math.exp(math.log(DESIRED_RES / BASE_RES) / (N_LEVELS - 1))


def level_layout(b=None):
    """Per level: (scale, resolution, table offset, table size, hashed).
    The scale 2^(l log2 b) 16 - 1 is evaluated in double from the float32
    log2 b and rounded once to float32 (the kernels' host code does the
    same, so both use identical scales)."""
    b = per_level_scale() if b is None else b
    log2b = float(np.float32(math.log2(float(np.float32(b)))))
    out, off = [], 0
    for lvl in range(N_LEVELS):
        scale = np.float32(2.0 ** (lvl * log2b) * BASE_RES - 1.0)
        res = int(math.ceil(float(scale))) + 1
        dense = res ** 3
        size = min(((dense + 7) // 8) * 8, 1 << LOG2_HASHMAP)
        out.append((float(scale), res, off, size, dense > size))
        off += size
    return out


def table_entries():
    lay = level_layout()
    return lay[-1][2] + lay[-1][3]


def grid_index(cell, res, size, hashed):
    """cell [..., 3] int64 -> entry index within the level's table."""
    if hashed:
        h = torch.zeros(cell.shape[:-1], dtype=torch.int64)
        for d in range(3):
            h = h ^ ((cell[..., d] * PRIMES[d]) & 0xFFFFFFFF)
        return h % size
    return (cell[..., 0] + cell[..., 1] * res + cell[..., 2] * res * res) % size


def encode(pos, table):
    """pos [N,3] in [0,1], table [entries, 2] -> features [N, 32]
    (feature index = level * 2 + f); differentiable in both."""
    feats = []
    for scale, res, off, size, hashed in level_layout():
        p = pos * scale + 0.5
        cell = torch.floor(p.detach())
        frac = p - cell
        cell = cell.to(torch.int64)
        acc = 0.0
        for corner in range(8):
            bit = torch.tensor([(corner >> d) & 1 for d in range(3)])
            w = torch.prod(torch.where(bit.bool(), frac, 1 - frac), dim=1, keepdim=True)
            idx = grid_index(cell + bit, res, size, hashed) + off
            acc = acc + w * table[idx]
        feats.append(acc)
    return torch.cat(feats, 1)


def mlp(x, weights):
    """Bias-free ReLU MLP: weights [W1 (32x32), W2 (32x32), W3 (Cx32)]
    (torch Linear layout, out x in)."""
    h = x
    for k, W in enumerate(weights):
        h = h @ W.T
        if k < len(weights) - 1:
            h = torch.relu(h)
    return h


class _ScaleGrad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, s):
        ctx.s = s
        return x.view_as(x)

    @staticmethod
    def backward(ctx, g):
        return g * ctx.s, None


def sample_noact(xyz, aabb, table, weights):
    """MLPTexture3D.sample_noact (geo/texture.py:101-112) with the hooks of
    :72-73 and :_MLP: the gradient into the encoding's output is scaled by
    128 (so the table's is), the gradient w.r.t. the positions is not."""
    t = (xyz.reshape(-1, 3) - aabb[0][None]) / (aabb[1] - aabb[0])[None]
    t = torch.clamp(t, min=0, max=1)
    t = _ScaleGrad.apply(t, 1.0 / GRADIENT_SCALING)
    enc = encode(t, table)
    enc = _ScaleGrad.apply(enc, GRADIENT_SCALING)
    return mlp(enc, weights)
