"""Host-side input checks of the drop-in, batched and serving entry points
(CPU only: every error here is raised before any device work)."""
import pytest
import torch

from dmgs_gb300.build import build
from dmgs_gb300.rasterizer import GaussianRasterizationSettings, GaussianRasterizer, check_inputs

P = 7


def settings(**kw):
    s = dict(image_height=32, image_width=48, tanfovx=0.5, tanfovy=0.4, bg=torch.zeros(3),
             scale_modifier=1.0, viewmatrix=torch.eye(4), projmatrix=torch.eye(4), sh_degree=3,
             campos=torch.zeros(3), prefiltered=False, debug=False)
    s.update(kw)
    return GaussianRasterizationSettings(**s)


def gaussians(**kw):
    g = dict(means3D=torch.zeros(P, 3), opacities=torch.zeros(P, 1), shs=torch.zeros(P, 16, 3),
             scales=torch.ones(P, 3), rotations=torch.zeros(P, 4))
    g.update(kw)
    return g


def test_reference_call_patterns_pass():
    check_inputs(**gaussians(), settings=[settings()])                     # stage 1 / config 1
    check_inputs(torch.zeros(P, 3), torch.zeros(P), colors_precomp=torch.zeros(P, 3),
                 cov3D_precomp=torch.zeros(P, 6), settings=[settings()])   # render_dyn (stage 2)
    check_inputs(**gaussians(shs=torch.zeros(P, 9, 3)))                    # fewer coefficients
    check_inputs(**gaussians(shs=torch.empty(0), means3D=torch.zeros(P, 3)))  # empty = absent
    check_inputs(torch.zeros(0, 3), torch.zeros(0, 1), shs=torch.zeros(0, 16, 3))  # P = 0


@pytest.mark.parametrize("kw,msg", [
    (dict(means3D=torch.zeros(P, 2)), "means3D must have dimensions"),
    (dict(means3D=torch.zeros(P * 3)), "means3D must have dimensions"),
    (dict(opacities=torch.zeros(P + 1)), "opacities must hold one value per point"),
    (dict(shs=torch.zeros(P, 3, 16)), "shs must have dimensions"),
    (dict(shs=torch.zeros(P - 1, 16, 3)), "shs must have dimensions"),
    (dict(scales=torch.zeros(P, 2)), "scales must have dimensions"),
    (dict(rotations=torch.zeros(P, 3)), "rotations must have dimensions"),
])
def test_bad_shapes_are_refused(kw, msg):
    with pytest.raises(RuntimeError, match=msg):
        check_inputs(**gaussians(**kw))


def test_bad_settings_are_refused():
    with pytest.raises(RuntimeError, match="viewmatrix must hold 16"):
        check_inputs(**gaussians(), settings=[settings(viewmatrix=torch.eye(3))])
    with pytest.raises(RuntimeError, match="bg must hold 3"):
        check_inputs(**gaussians(), settings=[settings(bg=torch.zeros(4))])


def test_drop_in_checks_shapes_then_refuses_cpu_tensors():
    build()
    rast = GaussianRasterizer(settings())
    g = gaussians()
    with pytest.raises(RuntimeError, match="cov3D_precomp must have dimensions"):
        rast(means3D=g["means3D"], means2D=torch.zeros(P, 3), opacities=g["opacities"],
             colors_precomp=torch.zeros(P, 3), cov3D_precomp=torch.zeros(P, 5))
    with pytest.raises(Exception, match="exactly one of either SHs"):
        rast(means3D=g["means3D"], means2D=torch.zeros(P, 3), opacities=g["opacities"],
             scales=g["scales"], rotations=g["rotations"])
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        rast(means3D=g["means3D"], means2D=torch.zeros(P, 3), opacities=g["opacities"],
             shs=g["shs"], scales=g["scales"], rotations=g["rotations"])


def test_batched_and_serving_entry_points_check_shapes():
    from dmgs_gb300.batched import BatchedRasterizer
    from dmgs_gb300.serving import ResidentScene
    with pytest.raises(RuntimeError, match="rotations must have dimensions"):
        BatchedRasterizer([settings()], gaussians(rotations=torch.zeros(P, 3)))
    with pytest.raises(RuntimeError, match="campos must hold 3"):
        BatchedRasterizer([settings(campos=torch.zeros(2))], gaussians())
    with pytest.raises(RuntimeError, match="shs must have dimensions"):
        ResidentScene(gaussians(shs=torch.zeros(P, 3, 16)))
