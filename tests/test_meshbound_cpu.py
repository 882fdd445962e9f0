"""Host-side pieces of the configuration-2 training step."""
import numpy as np

from dmgs_gb300.meshbound import eval_sh


def test_eval_sh_matches_the_oracle_polynomial():
    import torch
    from oracle import raster as R
    rng = np.random.default_rng(0)
    sh = rng.normal(0, 0.3, (50, 16, 3)).astype(np.float32)
    d = rng.normal(size=(50, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ours = eval_sh(3, torch.tensor(sh).permute(0, 2, 1), torch.tensor(d, dtype=torch.float32)).numpy()
    ref = R.eval_sh_rgb(3, sh.astype(np.float64), d)
    assert np.abs(ours + 0.5 - ref).max() < 1e-5  # the oracle adds the rasteriser offset


def test_sdf_regulariser_equals_the_mean_over_sign_changing_edges():
    """The masked-sum form (no host synchronisation) gives the value and
    gradient of the reference's form, which selects the sign-changing edges
    and takes the two BCE means (scene/gaussian_geo_model_mlp_flex.py:233-239)."""
    import torch
    import torch.nn.functional as F
    from dmgs_gb300.meshbound import sdf_reg_loss
    torch.manual_seed(0)
    for dt in (torch.float32, torch.float64):
        sdf = torch.randn(1000, dtype=dt, requires_grad=True)
        edges = torch.randint(0, 1000, (3000, 2))
        ours = sdf_reg_loss(sdf, edges)
        (g_ours,) = torch.autograd.grad(ours, sdf)
        s = sdf[edges.reshape(-1)].reshape(-1, 2)
        s = s[torch.sign(s[:, 0]) != torch.sign(s[:, 1])]
        ref = (F.binary_cross_entropy_with_logits(s[:, 0], (s[:, 1] > 0).to(dt)) +
               F.binary_cross_entropy_with_logits(s[:, 1], (s[:, 0] > 0).to(dt)))
        (g_ref,) = torch.autograd.grad(ref, sdf)
        tol = 1e-6 if dt == torch.float32 else 1e-12
        assert abs(ours.item() - ref.item()) <= tol * abs(ref.item())
        assert (g_ours - g_ref).abs().max().item() <= tol * g_ref.abs().max().item()
