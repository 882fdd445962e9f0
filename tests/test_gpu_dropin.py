"""The drop-in surface, driven the way the reference's renderer drives it.

``gaussian_renderer.render`` (gaussian_renderer/__init__.py:18-101) and
``render_dyn`` (:104-193) build a settings tuple, create a zero
``screenspace_points`` tensor that receives the screen-space gradient, and
call the rasteriser with keyword arguments; stage 2 passes precomputed
covariances and sigmoid(SH) colours computed in torch.  These tests follow
the same call sequence through ``import diff_gaussian_rasterization`` and
compare the autograd gradients with the oracle.
"""
import math

import numpy as np
import pytest
import torch

import dmgs_gb300
from dmgs_gb300.scenes import small_scene
from helpers import oracle_camera, rel_l2
from oracle import raster as R

pytestmark = pytest.mark.gpu


def _settings(mod, view, bg, deg, debug=False):
    d = "cuda"
    return mod.GaussianRasterizationSettings(
        image_height=int(view.height), image_width=int(view.width),
        tanfovx=math.tan(view.fovx * 0.5), tanfovy=math.tan(view.fovy * 0.5),
        bg=torch.tensor(bg, dtype=torch.float32, device=d), scale_modifier=1.0,
        viewmatrix=torch.tensor(view.viewmatrix, device=d),
        projmatrix=torch.tensor(view.projmatrix, device=d), sh_degree=deg,
        campos=torch.tensor(view.campos, device=d), prefiltered=False, debug=debug)


def test_render_stage1_pattern():
    mod = dmgs_gb300.install_as_diff_gaussian_rasterization()
    import diff_gaussian_rasterization as dgr
    assert dgr is mod
    sc = small_scene(P=4000, width=128, height=112, seed=21)
    view = sc.views[0]
    d = "cuda"
    xyz = torch.tensor(sc.means3D, device=d, requires_grad=True)
    opac = torch.tensor(sc.opacities, device=d, requires_grad=True)
    scales = torch.tensor(sc.scales, device=d, requires_grad=True)
    rots = torch.tensor(sc.rotations, device=d, requires_grad=True)
    shs = torch.tensor(sc.shs, device=d, requires_grad=True)
    screenspace_points = torch.zeros_like(xyz, dtype=xyz.dtype, requires_grad=True, device=d)
    screenspace_points.retain_grad()
    rast = dgr.GaussianRasterizer(raster_settings=_settings(dgr, view, [0, 0, 0], 3))
    img, radii = rast(means3D=xyz, means2D=screenspace_points, shs=shs, colors_precomp=None,
                      opacities=opac, scales=scales, rotations=rots, cov3D_precomp=None)
    assert img.shape == (3, 112, 128) and radii.dtype == torch.int32
    dimg = np.random.default_rng(0).standard_normal((3, 112, 128)).astype(np.float32)
    (img * torch.tensor(dimg, device=d)).sum().backward()

    cam = oracle_camera(view)
    ref = R.render(cam, sc.means3D, sc.opacities, shs=sc.shs, scales=sc.scales, rotations=sc.rotations)
    ok = ~ref.ambiguous
    assert np.abs(img.detach().cpu().numpy() - ref.image)[:, ok].max() <= 2e-4
    np.testing.assert_array_equal(radii.cpu().numpy(), ref.radii)
    go = ref.backward(dimg)
    pairs = {"means3D": xyz, "opacities": opac, "scales": scales, "rotations": rots, "shs": shs,
             "means2D": screenspace_points}
    for k, t in pairs.items():
        assert rel_l2(t.grad.cpu().numpy(), go[k]) <= 1e-3, k
    # the densification statistic reads the first two columns of means2D.grad
    assert torch.all(screenspace_points.grad[:, 2] == 0)


def test_render_dyn_stage2_pattern():
    """Precomputed covariance + sigmoid(SH) colours computed in torch."""
    import diff_gaussian_rasterization as dgr  # installed by the previous test or here
    dmgs_gb300.install_as_diff_gaussian_rasterization()
    sc = small_scene(P=3000, width=96, height=96, seed=22)
    view = sc.views[0]
    d = "cuda"
    xyz = torch.tensor(sc.means3D, device=d, requires_grad=True)
    cov_np = R.cov3d_from_scale_rot_f32(sc.scales, sc.rotations, 1.0).astype(np.float32)
    cov = torch.tensor(cov_np, device=d, requires_grad=True)
    feats = torch.tensor(sc.shs.transpose(0, 2, 1).copy(), device=d, requires_grad=True)  # [P,3,16]
    opac = torch.full((sc.P, 1), 0.9999, device=d)
    campos = torch.tensor(view.campos, device=d)
    dirs = xyz - campos.repeat(sc.P, 1)
    dirs = dirs / dirs.norm(dim=1, keepdim=True)
    sh2rgb = R.eval_sh_rgb(3, feats.transpose(1, 2), dirs) - 0.5
    colors = torch.sigmoid(sh2rgb)
    screenspace_points = torch.zeros_like(xyz, requires_grad=True)
    rast = dgr.GaussianRasterizer(raster_settings=_settings(dgr, view, [1, 1, 1], 3))
    img, radii = rast(means3D=xyz, means2D=screenspace_points, shs=None, colors_precomp=colors,
                      opacities=opac, scales=None, rotations=None, cov3D_precomp=cov)
    dimg = np.random.default_rng(1).standard_normal((3, 96, 96)).astype(np.float32)
    (img * torch.tensor(dimg, device=d)).sum().backward()

    # oracle on the same precomputed colours
    cam = oracle_camera(view, bg=(1, 1, 1))
    col_np = colors.detach().cpu().numpy()
    ref = R.render(cam, sc.means3D, opac.cpu().numpy(), colors=col_np, cov3D=cov_np)
    ok = ~ref.ambiguous
    assert np.abs(img.detach().cpu().numpy() - ref.image)[:, ok].max() <= 2e-4
    go = ref.backward(dimg)
    assert rel_l2(cov.grad.cpu().numpy(), go["cov3D_precomp"]) <= 1e-3
    # full chain to the SH features through torch autograd of the colour path
    col_t = torch.tensor(sc.means3D, dtype=torch.float64, requires_grad=True)
    f_t = torch.tensor(sc.shs.transpose(0, 2, 1).copy(), dtype=torch.float64, requires_grad=True)
    dd = col_t - torch.tensor(view.campos, dtype=torch.float64)
    dd = dd / dd.norm(dim=1, keepdim=True)
    c64 = torch.sigmoid(R.eval_sh_rgb(3, f_t.transpose(1, 2), dd) - 0.5)
    c64.backward(torch.tensor(go["colors_precomp"]))
    assert rel_l2(feats.grad.cpu().numpy(), f_t.grad.numpy()) <= 1e-3
    assert rel_l2(xyz.grad.cpu().numpy(), go["means3D"] + col_t.grad.numpy()) <= 1e-3


def test_input_mode_errors():
    import diff_gaussian_rasterization as dgr
    dmgs_gb300.install_as_diff_gaussian_rasterization()
    sc = small_scene(P=10, width=32, height=32)
    view = sc.views[0]
    d = "cuda"
    rast = dgr.GaussianRasterizer(raster_settings=_settings(dgr, view, [0, 0, 0], 3))
    xyz = torch.tensor(sc.means3D, device=d)
    m2 = torch.zeros_like(xyz)
    op = torch.tensor(sc.opacities, device=d)
    with pytest.raises(Exception):
        rast(means3D=xyz, means2D=m2, opacities=op, scales=torch.tensor(sc.scales, device=d),
             rotations=torch.tensor(sc.rotations, device=d))
    with pytest.raises(Exception):
        rast(means3D=xyz, means2D=m2, opacities=op, colors_precomp=torch.zeros(10, 3, device=d),
             scales=torch.tensor(sc.scales, device=d))
