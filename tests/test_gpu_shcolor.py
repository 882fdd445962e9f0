"""Fused sigmoid(SH) colour kernel (csrc/shcolor.cu through the C ABI)
against the float64 torch composition of the reference's Python path
(eval_sh on the normalised direction, then sigmoid; meshbound.eval_sh is
pinned to the reference's polynomial by tests/test_meshbound_cpu.py).

Tolerances: colours within 2e-6 absolute; gradients within 1e-5 relative L2
(float32 against float64)."""
import numpy as np
import pytest
import torch

from dmgs_gb300.meshbound import eval_sh

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float((a.double() - b.double()).norm() / b.double().norm().clamp_min(1e-30))


@pytest.mark.parametrize("deg,K", [(0, 16), (1, 16), (2, 16), (3, 16), (2, 9), (1, 7)])
def test_matches_torch_composition(deg, K):
    """K = 16: the 16-byte vector path; K = 9, 7: the scalar path."""
    from dmgs_gb300.shcolor import sh_colors
    g = torch.Generator().manual_seed(deg)
    P = 5000
    sh = torch.randn(P, 3, K, generator=g) * 0.5
    xyz = torch.randn(P, 3, generator=g) * 2.0
    campos = torch.tensor([0.3, -2.5, 4.0])
    up = torch.randn(P, 3, generator=g)
    s32 = sh.cuda().requires_grad_(True)
    x32 = xyz.cuda().requires_grad_(True)
    col = sh_colors(deg, s32, x32, campos.cuda())
    (col * up.cuda()).sum().backward()
    s64 = sh.double().requires_grad_(True)
    x64 = xyz.double().requires_grad_(True)
    d = x64 - campos.double()
    ref = torch.sigmoid(eval_sh(deg, s64, d / d.norm(dim=1, keepdim=True)))
    (ref * up.double()).sum().backward()
    assert (col.detach().cpu().double() - ref.detach()).abs().max() <= 2e-6
    assert rel_l2(s32.grad.cpu(), s64.grad) < 1e-5
    assert rel_l2(x32.grad.cpu(), x64.grad) < 1e-5 if deg > 0 else float(x32.grad.abs().max()) == 0.0
    nb = (deg + 1) ** 2
    assert float(s32.grad[:, :, nb:].abs().max() if nb < K else 0.0) == 0.0


def test_render_dyn_fused_equals_torch_colour():
    from dmgs_gb300.meshbound import MeshBoundScene, sphere_torus_mesh
    from dmgs_gb300.scenes import hemisphere_views
    v, f = sphere_torus_mesh(24)
    scene = MeshBoundScene(v, f, G=6, seed=0)
    view = hemisphere_views(1, 160, 120, seed=2)[0]
    bg = torch.zeros(3, device="cuda")
    a = scene.render(view, bg, fused_color=True)[0]
    b = scene.render(view, bg, fused_color=False)[0]
    assert float((a - b).detach().abs().max()) <= 1e-5


def test_rejects_bad_arguments():
    from dmgs_gb300.shcolor import sh_colors
    x = torch.zeros(4, 3, device="cuda")
    with pytest.raises(ValueError):
        sh_colors(3, torch.zeros(4, 3, 9, device="cuda"), x, torch.zeros(3, device="cuda"))
    with pytest.raises(ValueError):
        sh_colors(4, torch.zeros(4, 3, 25, device="cuda"), x, torch.zeros(3, device="cuda"))
