"""Configuration-2 training step on the GPU: binding -> SH colours ->
rasteriser (precomputed covariance and colours) -> L1 + SSIM; gradients
reach every parameter, are finite, and a few Adam steps lower the loss."""
import pytest
import torch

import numpy as np

from dmgs_gb300.meshbound import MeshBoundScene, sdf_sphere_torus, sphere_torus_mesh, training_step
from dmgs_gb300.scenes import hemisphere_views

pytestmark = pytest.mark.gpu


def test_configuration_mesh_is_closed_outward_with_the_reference_face_count():
    """FlexiCubes of the sphere-union-torus field at 64^3 (training mode):
    45,304 faces, every edge in two faces, normals along the SDF gradient."""
    v, f = sphere_torus_mesh(64)
    v, f = v.cpu().numpy().astype(np.float64), f.cpu().numpy()
    assert f.shape == (45304, 3) and f.min() >= 0 and f.max() < len(v)
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert np.all(counts == 2)
    c = v[f].mean(1)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    h = 1e-3
    grad = np.stack([(sdf_sphere_torus(c + h * np.eye(3)[i]) - sdf_sphere_torus(c - h * np.eye(3)[i]))
                     / (2 * h) for i in range(3)], 1)
    assert (((n * grad).sum(1) > 0).mean()) > 0.999
    assert np.abs(sdf_sphere_torus(v)).max() < 2.0 / 64


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


def test_stage2_full_step():
    """The reference's whole stage-2 iteration on the library's kernels:
    FlexiCubes every step -> binding -> hash-grid texture -> sigmoid(SH)
    colours -> rasteriser -> L1 + SSIM + SDF and FlexiCubes regularisers.
    Every learnable reaches a finite, non-zero gradient and a few Adam steps
    lower the loss."""
    from dmgs_gb300.meshbound import Stage2Model
    model = Stage2Model(res=32)
    views = hemisphere_views(3, 128, 128, seed=4)
    bg = torch.zeros(3, device="cuda")
    with torch.no_grad():
        saved = model.texture.encoder.params.clone()
        model.texture.encoder.params.add_(0.05 * torch.randn_like(saved))
        targets = [model.render(w, bg)[0].detach() for w in views]
        model.texture.encoder.params.copy_(saved)
    loss0 = model.step(views[0], targets[0], bg)
    assert torch.isfinite(loss0)
    for name, p in (("sdf", model.sdf), ("deform", model.deform),
                    ("per_cube_weights", model.per_cube_weights),
                    ("scale_factor", model.scale_factor),
                    ("texture", model.texture.encoder.params)):
        assert p.grad is not None and torch.isfinite(p.grad).all() and p.grad.abs().sum() > 0, name
    for w in model.texture.net.weights():
        assert torch.isfinite(w.grad).all() and w.grad.abs().sum() > 0
    opt = torch.optim.Adam([{"params": [model.texture.encoder.params], "lr": 1e-2},
                            {"params": list(model.texture.net.parameters()), "lr": 1e-3}])
    first = sum(float(model.step(w, t, bg)) for w, t in zip(views, targets))
    for _ in range(10):
        for w, t in zip(views, targets):
            model.step(w, t, bg)
            opt.step()
    last = sum(float(model.step(w, t, bg)) for w, t in zip(views, targets))
    assert last < first
