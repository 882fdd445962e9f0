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
