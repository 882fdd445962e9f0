"""The drop-in under the reference's own caller (CPU; needs the reference
tree, located through DMGS_REFERENCE_TREE, and skips without it).

The reference's gaussian_renderer (render, gaussian_renderer/__init__.py:
18-101; render_dyn, :104-193) is imported unmodified with this package
registered as ``diff_gaussian_rasterization``; its hard-coded CUDA device
use is redirected to the CPU and the third-party modules it imports but does
not use here are stubbed (as by the golden-vector generators).  The autograd
entry (``rasterize_gaussians``) is replaced by a recorder — there is no GPU
here — so the test checks everything the real caller hands the drop-in: the
settings NamedTuple (field by field), the keyword call, the input-mode
combinations of every pipeline switch, the shapes the kernels would index
(host-side checks), and that the screen-space gradient reaches the caller's
``viewspace_points`` tensor.
"""
import math
import os
import sys
import types

import pytest
import torch

REF = os.environ.get("DMGS_REFERENCE_TREE", "")
pytestmark = pytest.mark.skipif(
    not REF or not os.path.exists(os.path.join(REF, "gaussian_renderer", "__init__.py")),
    reason="reference tree not present (set DMGS_REFERENCE_TREE)")


@pytest.fixture(scope="module")
def ref_modules():
    from tests.golden.make_golden import CpuRedirect, install_stubs
    import dmgs_gb300
    from dmgs_gb300 import rasterizer
    saved = dict(sys.modules)
    install_stubs()
    dmgs_gb300.install_as_diff_gaussian_rasterization()
    sys.path.insert(0, REF)
    mode = CpuRedirect()
    mode.__enter__()
    try:
        import gaussian_renderer
        from scene.cameras import MiniCam
        from scene.gaussian_model import GaussianModel
        from utils.graphics_utils import getProjectionMatrix, getWorld2View2
        yield types.SimpleNamespace(renderer=gaussian_renderer, MiniCam=MiniCam,
                                    GaussianModel=GaussianModel, proj=getProjectionMatrix,
                                    w2v=getWorld2View2, rasterizer=rasterizer)
    finally:
        mode.__exit__(None, None, None)
        sys.path.remove(REF)
        for k in list(sys.modules):
            if k not in saved:
                del sys.modules[k]


class Recorder:
    """Stands in for the autograd entry: records the call, returns an image
    that depends on every tensor input (so autograd reaches them) and radii."""

    def __init__(self):
        self.calls = []

    def __call__(self, means3D, means2D, sh, colors_precomp, opacities, scales, rotations,
                 cov3Ds_precomp, raster_settings):
        args = dict(means3D=means3D, means2D=means2D, sh=sh, colors_precomp=colors_precomp,
                    opacities=opacities, scales=scales, rotations=rotations,
                    cov3Ds_precomp=cov3Ds_precomp, raster_settings=raster_settings)
        self.calls.append(args)
        H, W = raster_settings.image_height, raster_settings.image_width
        s = sum(t.sum() for t in args.values() if isinstance(t, torch.Tensor) and t.requires_grad)
        img = torch.zeros(3, H, W) + 0.0 * s
        radii = torch.ones(means3D.shape[0], dtype=torch.int32)
        return img, radii


def _camera(m, W=64, H=48, fovx=0.9):
    import numpy as np
    fovy = 2 * math.atan(math.tan(fovx / 2) * H / W)
    R = np.eye(3)
    T = np.array([0.1, -0.2, 4.0])
    wv = torch.tensor(m.w2v(R, T)).transpose(0, 1).float()
    pr = m.proj(znear=0.01, zfar=100.0, fovX=fovx, fovY=fovy).transpose(0, 1)
    full = (wv.unsqueeze(0).bmm(pr.unsqueeze(0))).squeeze(0)
    return m.MiniCam(W, H, fovy, fovx, 0.01, 100.0, wv, full)


def _model(m, P=200, deg=3):
    g = torch.Generator().manual_seed(0)
    pc = m.GaussianModel(deg)
    pc.active_sh_degree = deg
    pc._xyz = torch.randn(P, 3, generator=g).requires_grad_(True)
    pc._features_dc = torch.randn(P, 1, 3, generator=g).requires_grad_(True)
    pc._features_rest = (0.05 * torch.randn(P, (deg + 1) ** 2 - 1, 3, generator=g)).requires_grad_(True)
    pc._scaling = (torch.randn(P, 3, generator=g) - 4).requires_grad_(True)
    pc._rotation = torch.randn(P, 4, generator=g).requires_grad_(True)
    pc._opacity = torch.randn(P, 1, generator=g).requires_grad_(True)
    return pc


def _check_call(m, call, cam, P, bg, scaling_modifier=1.0):
    rs = call["raster_settings"]
    assert isinstance(rs, m.rasterizer.GaussianRasterizationSettings)
    assert rs._fields == ("image_height", "image_width", "tanfovx", "tanfovy", "bg",
                          "scale_modifier", "viewmatrix", "projmatrix", "sh_degree", "campos",
                          "prefiltered", "debug")
    assert (rs.image_height, rs.image_width) == (cam.image_height, cam.image_width)
    assert rs.tanfovx == pytest.approx(math.tan(cam.FoVx / 2))
    assert rs.tanfovy == pytest.approx(math.tan(cam.FoVy / 2))
    assert torch.equal(rs.viewmatrix, cam.world_view_transform)
    assert torch.equal(rs.projmatrix, cam.full_proj_transform)
    assert torch.equal(rs.campos, cam.camera_center)
    assert rs.bg is bg and rs.scale_modifier == scaling_modifier
    assert rs.prefiltered is False and rs.debug is False
    # the shapes the kernels index pass the drop-in's host-side checks
    m.rasterizer.check_inputs(call["means3D"], call["opacities"], call["sh"],
                              call["colors_precomp"], call["scales"], call["rotations"],
                              call["cov3Ds_precomp"], (rs,))
    assert call["means3D"].shape == (P, 3) and call["means2D"].shape == (P, 3)
    assert call["means2D"].requires_grad


@pytest.mark.parametrize("cov_py,sh_py", [(False, False), (True, False), (False, True), (True, True)])
def test_render_through_reference_caller(ref_modules, monkeypatch, cov_py, sh_py):
    m = ref_modules
    rec = Recorder()
    monkeypatch.setattr(m.rasterizer, "rasterize_gaussians", rec)
    cam = _camera(m)
    pc = _model(m)
    bg = torch.zeros(3)
    pipe = types.SimpleNamespace(debug=False, compute_cov3D_python=cov_py, convert_SHs_python=sh_py)
    out = m.renderer.render(cam, pc, pipe, bg, scaling_modifier=0.8)
    assert len(rec.calls) == 1
    call = rec.calls[0]
    _check_call(m, call, cam, 200, bg, 0.8)
    assert (call["sh"] is None) == sh_py and (call["colors_precomp"] is None) == (not sh_py)
    assert (call["cov3Ds_precomp"] is None) == (not cov_py)
    assert (call["scales"] is None) == cov_py and (call["rotations"] is None) == cov_py
    if not sh_py:
        assert call["sh"].shape == (200, 16, 3)
    if cov_py:
        assert call["cov3Ds_precomp"].shape == (200, 6)
    assert out["render"].shape == (3, 48, 64) and out["visibility_filter"].all()
    out["render"].sum().backward()
    assert out["viewspace_points"].grad is not None  # the caller's screen-space tensor


@pytest.mark.parametrize("sh_py", [True, False])
def test_render_dyn_through_reference_caller(ref_modules, monkeypatch, sh_py):
    m = ref_modules
    rec = Recorder()
    monkeypatch.setattr(m.rasterizer, "rasterize_gaussians", rec)
    cam = _camera(m)
    P = 120
    g = torch.Generator().manual_seed(1)
    gs = {"xyz": torch.randn(P, 3, generator=g).requires_grad_(True),
          "opacity": torch.rand(P, 1, generator=g).requires_grad_(True),
          "covariance": (1e-3 * torch.rand(P, 6, generator=g)).requires_grad_(True),
          "features": torch.randn(P, 3, 16, generator=g).requires_grad_(True),
          "active_sh_degree": 3, "max_sh_degree": 3}
    bg = torch.ones(3)
    pipe = types.SimpleNamespace(debug=False, compute_cov3D_python=True, convert_SHs_python=sh_py)
    out = m.renderer.render_dyn(cam, gs, pipe, bg)
    call = rec.calls[0]
    assert call["cov3Ds_precomp"] is gs["covariance"] and call["scales"] is None
    if not sh_py:
        # render_dyn then hands over the stage-2 features as they are,
        # [P, 3, 16] channel-major, where the rasteriser's SH input is
        # [P, M, 3]; the reference's stage-2 scripts never take this branch
        # (they force convert_SHs_python, train_geo_stage2.py:268-269).  The
        # drop-in refuses the layout on the host instead of reading it wrongly.
        assert call["colors_precomp"] is None and call["sh"] is gs["features"]
        with pytest.raises(RuntimeError, match=r"shs must have dimensions \(num_points, M, 3\)"):
            _check_call(m, call, cam, P, bg)
        return
    _check_call(m, call, cam, P, bg)
    assert call["sh"] is None and call["colors_precomp"].shape == (P, 3)
    out["render"].sum().backward()
    assert out["viewspace_points"].grad is not None and gs["xyz"].grad is not None


def test_input_mode_errors_reach_the_caller(ref_modules, monkeypatch):
    """override_color together with SH conversion off still passes exactly
    one colour source; the drop-in raises the reference's exception when a
    caller passes both (its own error text)."""
    m = ref_modules
    rec = Recorder()
    monkeypatch.setattr(m.rasterizer, "rasterize_gaussians", rec)
    cam = _camera(m)
    pc = _model(m)
    pipe = types.SimpleNamespace(debug=False, compute_cov3D_python=False, convert_SHs_python=False)
    m.renderer.render(cam, pc, pipe, torch.zeros(3), override_color=torch.rand(200, 3))
    assert rec.calls[0]["sh"] is None and rec.calls[0]["colors_precomp"].shape == (200, 3)
    rs = rec.calls[0]["raster_settings"]
    with pytest.raises(Exception, match="exactly one of either SHs or precomputed colors"):
        m.rasterizer.GaussianRasterizer(rs)(means3D=pc.get_xyz, means2D=torch.zeros(200, 3),
                                            opacities=pc.get_opacity, shs=pc.get_features,
                                            colors_precomp=torch.rand(200, 3),
                                            scales=pc.get_scaling, rotations=pc.get_rotation)
