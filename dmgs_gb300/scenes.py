"""Seeded synthetic scenes with the shapes and value distributions of the
benchmark workloads (the reference's datasets — NeRF-Synthetic and
Mip-NeRF360 — are not available; these stand in for them).

All generators use numpy's PCG64 (platform-independent), return float32
arrays in the reference's layouts (means [P,3], scales [P,3], quaternions
[P,4] (r,x,y,z), opacities [P,1], SH [P,16,3] coefficient-major) and a
:class:`dmgs_gb300.camera.ViewSpec`.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .camera import ViewSpec, make_view


@dataclass
class Scene:
    means3D: np.ndarray
    scales: np.ndarray
    rotations: np.ndarray
    opacities: np.ndarray
    shs: np.ndarray
    views: list = field(default_factory=list)
    sh_degree: int = 3

    @property
    def P(self):
        return self.means3D.shape[0]


def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def _unit_quats(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def _shs(rng, n, dc_mean=0.5, dc_std=0.2, rest_std=0.05, coeffs=16):
    sh = np.empty((n, coeffs, 3), np.float32)
    sh[:, 0, :] = rng.normal(dc_mean, dc_std, (n, 3))
    sh[:, 1:, :] = rng.normal(0.0, rest_std, (n, coeffs - 1, 3))
    return sh


def small_scene(P=10_000, width=256, height=256, fov_deg=50.0, seed=0):
    """Plain-rasteriser workload: P Gaussians uniform in [-1,1]^3, scales
    exp(U(-5,-3)), uniform unit quaternions, opacity sigmoid(N(0,1)), SH
    degree 3 (DC ~ N(0.5,0.2), rest ~ N(0,0.05)); one camera at radius 4
    looking at the origin."""
    rng = np.random.default_rng(seed)
    means = rng.uniform(-1.0, 1.0, (P, 3)).astype(np.float32)
    scales = np.exp(rng.uniform(-5.0, -3.0, (P, 3))).astype(np.float32)
    rots = _unit_quats(rng, P)
    opac = _sigmoid(rng.standard_normal((P, 1))).astype(np.float32)
    shs = _shs(rng, P)
    az, el = math.radians(30.0), math.radians(20.0)
    eye = 4.0 * np.array([math.sin(az) * math.cos(el), math.sin(el), math.cos(az) * math.cos(el)])
    view = make_view(eye, (0.0, 0.0, 0.0), width, height, fovx_deg=fov_deg)
    return Scene(means, scales, rots, opac, shs, [view])


def large_scene(P=3_000_000, seed=0, n_views=1, width=1237, height=822, fov_deg=60.0,
                resolutions=None):
    """Large-scene workload: 90% of the means from 64 isotropic clusters
    (sigma ~ U(0.2,1.5), centres uniform in the ball of radius 5), 10% on a
    background shell of radius U(20,40); scales log-normal(-4,1); opacity
    sigmoid(N(0,1.5)); SH degree 3.  Views: camera inside radius 3 looking
    outward (horizontally) at a random yaw, FoV 60 degrees horizontal.
    `resolutions`: optional list of (width, height) assigned round-robin."""
    rng = np.random.default_rng(seed)
    n_fg = int(round(P * 0.9))
    n_bg = P - n_fg
    centres = rng.standard_normal((64, 3))
    centres /= np.linalg.norm(centres, axis=1, keepdims=True)
    centres *= 5.0 * rng.uniform(0, 1, (64, 1)) ** (1.0 / 3.0)
    sig = rng.uniform(0.2, 1.5, 64)
    which = rng.integers(0, 64, n_fg)
    fg = centres[which] + rng.standard_normal((n_fg, 3)) * sig[which, None]
    d = rng.standard_normal((n_bg, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    bg = d * rng.uniform(20.0, 40.0, (n_bg, 1))
    means = np.concatenate([fg, bg], 0).astype(np.float32)
    perm = rng.permutation(P)
    means = means[perm]
    scales = np.exp(rng.normal(-4.0, 1.0, (P, 3))).astype(np.float32)
    rots = _unit_quats(rng, P)
    opac = _sigmoid(rng.normal(0.0, 1.5, (P, 1))).astype(np.float32)
    shs = _shs(rng, P)
    views = []
    for v in range(n_views):
        w, h = (width, height) if resolutions is None else resolutions[v % len(resolutions)]
        views.append(random_inside_view(rng, w, h, fov_deg))
    return Scene(means, scales, rots, opac, shs, views)


def random_inside_view(rng, width, height, fov_deg=60.0, radius=3.0):
    """Camera uniformly inside the ball of `radius`, looking outward
    horizontally at a random yaw."""
    p = rng.standard_normal(3)
    p = p / np.linalg.norm(p) * radius * rng.uniform(0, 1) ** (1.0 / 3.0)
    yaw = rng.uniform(0, 2 * math.pi)
    fwd = np.array([math.cos(yaw), 0.0, math.sin(yaw)])
    return make_view(p, p + fwd, width, height, fovx_deg=fov_deg)


def hemisphere_views(n, width, height, radius=4.0, fov_deg=50.0, seed=0):
    """`n` cameras uniform on the upper hemisphere (y > 0) at `radius`,
    looking at the origin."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        d = rng.standard_normal(3)
        d[1] = abs(d[1])
        d /= np.linalg.norm(d)
        out.append(make_view(radius * d, (0.0, 0.0, 0.0), width, height, fovx_deg=fov_deg))
    return out


def large_scene_tensors(P, seed, device):
    """The large-scene distributions of :func:`large_scene`, generated on
    `device` with torch's generator (for the many-million-Gaussian resident
    scenes of the serving workload; a different random stream than the
    numpy generator).  Returns a dict of contiguous fp32 tensors with the
    reference's names (means3D, scales, rotations, opacities, shs)."""
    import torch

    g = torch.Generator(device=device).manual_seed(int(seed))
    f = dict(device=device, dtype=torch.float32, generator=g)
    n_fg = int(round(P * 0.9))
    n_bg = P - n_fg
    centres = torch.randn(64, 3, **f)
    centres = centres / centres.norm(dim=1, keepdim=True)
    centres = centres * 5.0 * torch.rand(64, 1, **f) ** (1.0 / 3.0)
    sig = 0.2 + 1.3 * torch.rand(64, **f)
    which = torch.randint(0, 64, (n_fg,), device=device, generator=g)
    fg = centres[which] + torch.randn(n_fg, 3, **f) * sig[which, None]
    d = torch.randn(n_bg, 3, **f)
    d = d / d.norm(dim=1, keepdim=True)
    bg = d * (20.0 + 20.0 * torch.rand(n_bg, 1, **f))
    means = torch.cat([fg, bg], 0)[torch.randperm(P, device=device, generator=g)]
    q = torch.randn(P, 4, **f)
    sh = torch.empty(P, 16, 3, device=device)
    sh[:, 0, :] = 0.5 + 0.2 * torch.randn(P, 3, **f)
    sh[:, 1:, :] = 0.05 * torch.randn(P, 15, 3, **f)
    return {"means3D": means.contiguous(),
            "scales": torch.exp(-4.0 + torch.randn(P, 3, **f)).contiguous(),
            "rotations": (q / q.norm(dim=1, keepdim=True)).contiguous(),
            "opacities": torch.sigmoid(1.5 * torch.randn(P, 1, **f)).contiguous(),
            "shs": sh.contiguous()}
