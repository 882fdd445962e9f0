"""Configuration-2 training step on the GPU: binding -> SH colours ->
rasteriser (precomputed covariance and colours) -> L1 + SSIM; gradients
reach every parameter, are finite, and a few Adam steps lower the loss."""
import pytest
import torch

from dmgs_gb300.meshbound import MeshBoundScene, sphere_torus_mesh, training_step
from dmgs_gb300.scenes import hemisphere_views

pytestmark = pytest.mark.gpu


def test_training_step_gradients_and_descent():
    v, f = sphere_torus_mesh(24)
    scene = MeshBoundScene(v, f, G=6, seed=0)
    target = MeshBoundScene(v, f, G=6, seed=0)
    with torch.no_grad():
        target.verts.add_(0.01 * torch.randn_like(target.verts))
        target.features.add_(0.1 * torch.randn_like(target.features))
    views = hemisphere_views(4, 128, 128, seed=1)
    bg = torch.zeros(3, device="cuda")
    targets = [target.render(w, bg)[0].detach() for w in views]
    loss0, radii = training_step(scene, views[0], targets[0], bg)
    assert torch.isfinite(loss0) and (radii > 0).sum() > 100
    for p in scene.params():
        assert p.grad is not None and torch.isfinite(p.grad).all() and p.grad.abs().sum() > 0
    opt = torch.optim.Adam(scene.params(), lr=1e-3)
    first = sum(float(training_step(scene, w, t, bg)[0]) for w, t in zip(views, targets))
    for _ in range(15):
        for w, t in zip(views, targets):
            training_step(scene, w, t, bg)
            opt.step()
    last = sum(float(training_step(scene, w, t, bg)[0]) for w, t in zip(views, targets))
    assert last < first
