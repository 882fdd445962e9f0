"""Mesh-bound Gaussian training step (the stage-2 path of the reference).

The reference's stage-2 step (train_geo_stage2.py:101-116) extracts a mesh
(FlexiCubes), binds Gaussians to its faces (renew_gaussian /
get_covariance_dyn, scene/gaussian_geo_model_mlp_flex.py:258-335,370-385),
evaluates SH colours in torch (gaussian_renderer/__init__.py:165-170:
eval_sh then sigmoid), rasterises with precomputed covariance and colours
(render_dyn, :104-193) and optimises L1 + 0.2 (1 - SSIM)
(utils/loss_utils.py).  Here the binding, the SH colour (sigmoid of
eval_sh), the rasteriser and the loss are this library's kernels; the torch
compositions of the colour and the loss remain selectable
(``fused_color=False``, ``fused_loss=False``) as the reference's form.

The mesh of the workload is built by :func:`sphere_torus_mesh`: this
library's FlexiCubes extraction (csrc/flexicubes.cu) of the union of a
sphere (r 0.6) and a torus (R 0.7, r 0.2) sampled on a 64^3 grid over
[-1, 1]^3, in training mode (45,304 faces).
"""
from __future__ import annotations

import math

import numpy as np
import torch
import torch.nn.functional as F_

from .binding import bind_faces
from .flexicubes import FlexiCubes
from .loss import l1_ssim_loss
from .shcolor import sh_colors
from .rasterizer import GaussianRasterizationSettings, GaussianRasterizer

# Real SH basis constants (degree <= 3), the standard orthonormal basis.
_C0 = 0.28209479177387814
_C1 = 0.4886025119029199
_C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792,
       0.5462742152960396)
_C3 = (-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154,
       -0.4570457994644658, 1.445305721320277, -0.5900435899266435)


def sdf_sphere_torus(p):
    sph = np.linalg.norm(p, axis=-1) - 0.6
    q = np.sqrt(p[..., 0] ** 2 + p[..., 2] ** 2) - 0.7
    tor = np.sqrt(q ** 2 + p[..., 1] ** 2) - 0.2
    return np.minimum(sph, tor)


def sphere_torus_mesh(res=64, lo=-1.0, hi=1.0, sdf=sdf_sphere_torus, device="cuda"):
    """FlexiCubes extraction (training mode, uniform weights, undeformed
    grid) of an SDF sampled on a res^3 grid over [lo, hi]^3, on the device:
    (verts [V,3] float32, faces [F,3] int64), consistently outward.  For the
    sphere-union-torus field at 64^3 that is 45,304 faces."""
    fc = FlexiCubes(device=device)
    grid, cubes = fc.construct_voxel_grid_v2(res, [lo] * 3, [hi] * 3)
    s = torch.as_tensor(sdf(grid.double().cpu().numpy()), dtype=torch.float32, device=device)
    v, f, _, _ = fc(grid, s, cubes, res, training=True)
    return v.detach(), f


def eval_sh(deg, sh, dirs):
    """SH colour (degree <= 3) of features sh [P, 3, (deg+1)^2] at unit
    directions dirs [P, 3] (the real SH polynomial of the 3DGS reference,
    utils/sh_utils.py:25-110)."""
    x, y, z = dirs[:, 0:1], dirs[:, 1:2], dirs[:, 2:3]
    r = _C0 * sh[..., 0]
    if deg > 0:
        r = r - _C1 * y * sh[..., 1] + _C1 * z * sh[..., 2] - _C1 * x * sh[..., 3]
        if deg > 1:
            xx, yy, zz, xy, yz, xz = x * x, y * y, z * z, x * y, y * z, x * z
            r = (r + _C2[0] * xy * sh[..., 4] + _C2[1] * yz * sh[..., 5]
                 + _C2[2] * (2.0 * zz - xx - yy) * sh[..., 6] + _C2[3] * xz * sh[..., 7]
                 + _C2[4] * (xx - yy) * sh[..., 8])
            if deg > 2:
                r = (r + _C3[0] * y * (3 * xx - yy) * sh[..., 9] + _C3[1] * xy * z * sh[..., 10]
                     + _C3[2] * y * (4 * zz - xx - yy) * sh[..., 11]
                     + _C3[3] * z * (2 * zz - 3 * xx - 3 * yy) * sh[..., 12]
                     + _C3[4] * x * (4 * zz - xx - yy) * sh[..., 13]
                     + _C3[5] * z * (xx - yy) * sh[..., 14]
                     + _C3[6] * x * (xx - 3 * yy) * sh[..., 15])
    return r


def _gauss_window(size=11, sigma=1.5, channels=3, device="cuda", dtype=torch.float32):
    g = torch.exp(-((torch.arange(size, device=device, dtype=dtype) - size // 2) ** 2)
                  / (2 * sigma ** 2))
    g = g / g.sum()
    w = (g[:, None] * g[None, :])[None, None]
    return w.expand(channels, 1, size, size).contiguous()


def ssim(img1, img2, window=None):
    """Mean SSIM (Wang et al. 2004) with an 11x11 Gaussian window (sigma 1.5),
    C1 = 0.01^2, C2 = 0.03^2, per channel — the form of the reference's
    utils/loss_utils.py."""
    C = img1.shape[0]
    w = window if window is not None else _gauss_window(channels=C, device=img1.device,
                                                        dtype=img1.dtype)
    a, b = img1[None], img2[None]
    mu1 = F_.conv2d(a, w, padding=5, groups=C)
    mu2 = F_.conv2d(b, w, padding=5, groups=C)
    s11 = F_.conv2d(a * a, w, padding=5, groups=C) - mu1 * mu1
    s22 = F_.conv2d(b * b, w, padding=5, groups=C) - mu2 * mu2
    s12 = F_.conv2d(a * b, w, padding=5, groups=C) - mu1 * mu2
    C1, C2 = 0.01 ** 2, 0.03 ** 2
    m = ((2 * mu1 * mu2 + C1) * (2 * s12 + C2)) / ((mu1 * mu1 + mu2 * mu2 + C1) * (s11 + s22 + C2))
    return m.mean()



def view_tensors(view, device, cache):
    """(camera centre, view matrix, projection matrix) of `view` on the
    device, uploaded once per view and kept in `cache` — as the reference's
    Camera holds them on the device (scene/cameras.py:54-57).  An upload per
    step from host memory would wait for the work already queued on the GPU."""
    hit = cache.get(id(view))
    if hit is None or hit[0] is not view:
        hit = (view, torch.tensor(view.campos, device=device),
               torch.tensor(view.viewmatrix, device=device),
               torch.tensor(view.projmatrix, device=device))
        cache[id(view)] = hit
    return hit[1:]

class MeshBoundScene:
    """Gaussians bound to a mesh's faces (stage 2): learnable vertices and
    scale factor, G Gaussians per face at per-Gaussian Dirichlet(1,1,1)
    barycentric coordinates, per-Gaussian SH features [P, 3, 16] and
    opacities."""

    def __init__(self, verts, faces, G=6, seed=0, device="cuda", sh_degree=3):
        rng = np.random.default_rng(seed)
        self.device = torch.device(device)
        self.faces = torch.as_tensor(faces, device=self.device)
        F = self.faces.shape[0]
        self.G, self.P = G, F * G
        self.verts = torch.as_tensor(verts, dtype=torch.float32, device=self.device).detach().clone()
        self.verts.requires_grad_(True)
        self.bc = torch.tensor(rng.dirichlet((1.0, 1.0, 1.0), (F, G)).astype(np.float32),
                               device=self.device)
        self.rad_base = 1.0 / (4.0 + 2.0 * math.sqrt(3.0))
        self.max_scale = 2.0  # the reference's initial scale factor: atanh(1 / max_scale)
        self.scale_factor = torch.full((1,), math.atanh(1.0 / self.max_scale), device=self.device,
                                       requires_grad=True)
        sh = np.zeros((self.P, 3, 16), np.float32)
        sh[:, :, 0] = rng.normal(0.5, 0.2, (self.P, 3))
        sh[:, :, 1:] = rng.normal(0.0, 0.05, (self.P, 3, 15))
        self.features = torch.tensor(sh, device=self.device, requires_grad=True)
        self.opacity = torch.tensor(
            (1.0 / (1.0 + np.exp(-rng.standard_normal((self.P, 1))))).astype(np.float32),
            device=self.device, requires_grad=True)
        self.sh_degree = sh_degree
        self.spatial_lr_scale = 1.0
        self._views = {}

    def params(self):
        return [self.verts, self.scale_factor, self.features, self.opacity]

    def gaussians(self):
        xyz, cov, _ = bind_faces(self.verts, self.faces, self.bc, self.scale_factor,
                                 self.rad_base, self.spatial_lr_scale, self.max_scale)
        return xyz, cov

    def render(self, view, bg, fused_color=True):
        """render_dyn: precomputed covariance and sigmoid(SH) colours (the
        fused colour kernel, or the torch composition with fused_color=False)."""
        xyz, cov = self.gaussians()
        campos, viewm, projm = view_tensors(view, self.device, self._views)
        if fused_color:
            colors = sh_colors(self.sh_degree, self.features, xyz, campos)
        else:
            d = xyz - campos
            d = d / d.norm(dim=1, keepdim=True)
            colors = torch.sigmoid(eval_sh(self.sh_degree, self.features, d))
        rs = GaussianRasterizationSettings(
            image_height=view.height, image_width=view.width, tanfovx=view.tanfovx,
            tanfovy=view.tanfovy, bg=bg, scale_modifier=1.0, viewmatrix=viewm, projmatrix=projm,
            sh_degree=self.sh_degree, campos=campos, prefiltered=False, debug=False)
        means2D = torch.zeros_like(xyz, requires_grad=True)
        img, radii = GaussianRasterizer(rs)(means3D=xyz, means2D=means2D, opacities=self.opacity,
                                            colors_precomp=colors, cov3D_precomp=cov)
        return img, radii, means2D


def training_step(scene: MeshBoundScene, view, target, bg, lambda_dssim=0.2, window=None,
                  fused_loss=True, fused_color=True):
    """One stage-2 step, forward and backward: bind, colour, rasterise,
    L1 + lambda (1 - SSIM) (the fused kernels, or the torch compositions with
    fused_loss=False / fused_color=False), gradients into the scene's
    parameters."""
    for p in scene.params():
        p.grad = None
    img, radii, _ = scene.render(view, bg, fused_color=fused_color)
    if fused_loss:
        loss = l1_ssim_loss(img, target, lambda_dssim)
    else:
        loss = (1.0 - lambda_dssim) * (img - target).abs().mean() + lambda_dssim * (
            1.0 - ssim(img, target, window))
    loss.backward()
    return loss.detach(), radii


def sdf_reg_loss(sdf, edges):
    """The reference's SDF regulariser (compute_sdf_reg_loss,
    scene/gaussian_geo_model_mlp_flex.py:233-239): binary cross-entropy of
    each sign-changing edge's end values against the other end's sign."""
    s = sdf[edges.reshape(-1)].reshape(-1, 2)
    # the means over the sign-changing edges as masked sums: no host
    # synchronisation for the selection's size
    m = (torch.sign(s[:, 0]) != torch.sign(s[:, 1])).to(s.dtype)
    n = m.sum()
    bce = F_.binary_cross_entropy_with_logits
    return ((bce(s[:, 0], (s[:, 1] > 0).to(s.dtype), reduction="none") * m).sum() / n +
            (bce(s[:, 1], (s[:, 0] > 0).to(s.dtype), reduction="none") * m).sum() / n)


class Stage2Model:
    """The reference's stage-2 model and iteration on this library's kernels
    (scene/gaussian_geo_model_mlp_flex.py with train_geo_stage2.py:101-135):
    a FlexiCubes grid with learnable SDF, deformation and per-cube weights,
    extracted every step in training mode (getMesh, :241-255); Gaussians
    bound to the faces with the shared barycentric table (renew_gaussian,
    :258-335, opacity 0.9999); SH features from the hash-grid texture (:313);
    sigmoid(SH) colours; the rasteriser with precomputed covariance and
    colours (render_dyn); loss (1 - l) L1 + l (1 - SSIM) + lambda_sdf
    sdf_reg + lambda_flex mean(L_dev) (the defaults of
    arguments/__init__.py:112-114)."""

    def __init__(self, res=64, gs_per_face=6, device="cuda", sdf=sdf_sphere_torus, sh_degree=3):
        from .binding import barycentric_table
        from .texture import MLPTexture3D
        self.device = torch.device(device)
        self.res = res
        self.fc = FlexiCubes(device=device)
        self.grid, self.cubes = self.fc.construct_voxel_grid_v2(res, [-1.0] * 3, [1.0] * 3)
        self.sdf = torch.as_tensor(sdf(self.grid.double().cpu().numpy()), dtype=torch.float32,
                                   device=self.device).requires_grad_(True)
        self.deform = torch.zeros_like(self.grid, requires_grad=True)
        self.per_cube_weights = torch.ones((self.cubes.shape[0], 21), device=self.device,
                                           requires_grad=True)
        self.max_displacement = (2.0 / res) / 4.0
        self.bc, self.rad_base = barycentric_table(gs_per_face, device)
        self.max_scale = 2.0
        self.scale_factor = torch.full((1,), math.atanh(1.0 / self.max_scale), device=self.device,
                                       requires_grad=True)
        self.spatial_lr_scale = 1.0
        self.sh_degree = sh_degree
        self._views = {}
        with torch.no_grad():
            v = self.mesh()[0]
            aabb = torch.stack([v.min(0).values, v.max(0).values]) * 1.1
        self.texture = MLPTexture3D(aabb, channels=3 * (sh_degree + 1) ** 2, device=device)

    def params(self):
        return [self.sdf, self.deform, self.per_cube_weights, self.scale_factor] + list(
            self.texture.parameters())

    def mesh(self):
        v = self.grid + self.max_displacement * torch.tanh(self.deform)
        w = self.per_cube_weights
        return self.fc(v, self.sdf, self.cubes, self.res, w[:, :12], w[:, 12:20], w[:, 20],
                       training=True)

    def render(self, view, bg):
        verts, faces, L_dev, surf_edges = self.mesh()
        xyz, cov, _ = bind_faces(verts, faces, self.bc, self.scale_factor, self.rad_base,
                                 self.spatial_lr_scale, self.max_scale)
        K = (self.sh_degree + 1) ** 2
        feats = self.texture.sample_noact(xyz).view(-1, 3, K)
        campos, viewm, projm = view_tensors(view, self.device, self._views)
        colors = sh_colors(self.sh_degree, feats, xyz, campos)
        rs = GaussianRasterizationSettings(
            image_height=view.height, image_width=view.width, tanfovx=view.tanfovx,
            tanfovy=view.tanfovy, bg=bg, scale_modifier=1.0, viewmatrix=viewm, projmatrix=projm,
            sh_degree=self.sh_degree, campos=campos, prefiltered=False, debug=False)
        opac = torch.full((xyz.shape[0], 1), 0.9999, device=self.device)
        img, radii = GaussianRasterizer(rs)(
            means3D=xyz, means2D=torch.zeros_like(xyz, requires_grad=True), opacities=opac,
            colors_precomp=colors, cov3D_precomp=cov)
        return img, radii, L_dev, surf_edges

    def step(self, view, target, bg, lambda_dssim=0.2, lambda_sdf=0.2, lambda_flex=0.25):
        """One iteration's forward and backward; returns the loss."""
        for p in self.params():
            p.grad = None
        img, radii, L_dev, surf_edges = self.render(view, bg)
        loss = (l1_ssim_loss(img, target, lambda_dssim) + lambda_sdf * sdf_reg_loss(self.sdf, surf_edges)
                + lambda_flex * L_dev.mean())
        loss.backward()
        return loss.detach()
