"""The fused L1 + SSIM kernels against the torch composition of the same
loss (float64 reference): value and gradient, odd image sizes, zero and
identical inputs."""
import pytest
import torch

from dmgs_gb300.loss import l1_ssim_loss
from dmgs_gb300.meshbound import ssim

pytestmark = pytest.mark.gpu


def _torch_loss(x, y, lam):
    return (1 - lam) * (x - y).abs().mean() + lam * (1 - ssim(x, y))


@pytest.mark.parametrize("shape", [(3, 64, 64), (3, 97, 131), (1, 17, 300), (3, 800, 800)])
def test_value_and_gradient_match_torch(shape):
    g = torch.Generator(device="cuda").manual_seed(sum(shape))
    y = torch.rand(shape, device="cuda", generator=g)
    x = (y + 0.1 * torch.randn(shape, device="cuda", generator=g)).clamp(0, 1)
    xd = x.double().requires_grad_(True)
    ref = _torch_loss(xd, y.double(), 0.2)
    ref.backward()
    xf = x.clone().requires_grad_(True)
    ours = l1_ssim_loss(xf, y, 0.2)
    ours.backward()
    r = float(ref.detach())
    assert abs(float(ours.detach()) - r) <= 1e-5 * max(1.0, abs(r))
    rel = (xf.grad.double() - xd.grad).norm() / xd.grad.norm()
    assert rel <= 1e-4


def test_identical_images_have_zero_loss_and_l1_free_gradient():
    x = torch.rand(3, 40, 50, device="cuda")
    xr = x.clone().requires_grad_(True)
    loss = l1_ssim_loss(xr, x, 0.2)
    loss.backward()
    assert abs(float(loss.detach())) < 1e-5
    assert xr.grad.abs().max() < 1e-6  # SSIM is stationary there, sign(0) = 0


def test_matches_the_reference_loss_golden_vectors():
    """The fused kernels against golden vectors from the reference's own
    utils/loss_utils.py (l1_loss and ssim as train_geo_stage2.py:114-116
    combines them, float64 on the CPU): value to 1e-5 relative, gradient
    to 1e-4 relative L2 (float32 kernels)."""
    import os
    import numpy as np
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "loss_golden.npz"))
    for i in range(int(z["n"])):
        x = torch.tensor(z[f"x{i}"], device="cuda", requires_grad=True)
        y = torch.tensor(z[f"y{i}"], device="cuda")
        loss = l1_ssim_loss(x, y, float(z[f"lam{i}"]))
        loss.backward()
        ref = float(z[f"loss{i}"])
        assert abs(loss.item() - ref) <= 1e-5 * max(1.0, abs(ref))
        g = z[f"grad{i}"].astype(np.float64)
        assert np.linalg.norm(x.grad.double().cpu().numpy() - g) <= 1e-4 * np.linalg.norm(g)
