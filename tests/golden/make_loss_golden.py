"""Golden vectors for the fused L1 + SSIM loss from the reference's own
``utils/loss_utils.py`` (``l1_loss``, ``ssim``), combined as the stage-2
training loop does (train_geo_stage2.py:114-116):
``(1 - lambda) * l1_loss(image, gt) + lambda * (1 - ssim(image, gt))``,
run on the CPU in float64 on float32 image pairs.

    python tests/golden/make_loss_golden.py [/path/to/reference]

Output: ``loss_golden.npz``: per case the two images [C, H, W] (float32),
lambda, the loss (float64) and its gradient w.r.t. the first image (stored
as float32).
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [((3, 40, 50), 0.2), ((1, 17, 33), 0.2), ((3, 23, 64), 0.5)]


def main(ref):
    sys.path.insert(0, ref)
    from utils.loss_utils import l1_loss, ssim
    out = {}
    for i, (shape, lam) in enumerate(CASES):
        rng = np.random.default_rng(100 + i)
        y = rng.uniform(0, 1, shape).astype(np.float32)
        x = np.clip(y + rng.normal(0, 0.1, shape), 0, 1).astype(np.float32)
        xt = torch.tensor(x, dtype=torch.float64, requires_grad=True)
        yt = torch.tensor(y, dtype=torch.float64)
        loss = (1.0 - lam) * l1_loss(xt, yt) + lam * (1.0 - ssim(xt, yt))
        loss.backward()
        out[f"x{i}"], out[f"y{i}"] = x, y
        out[f"lam{i}"] = np.float64(lam)
        out[f"loss{i}"] = np.float64(loss.item())
        out[f"grad{i}"] = xt.grad.numpy().astype(np.float32)  # float32 suffices for the test bars
        print(shape, lam, loss.item())
    np.savez_compressed(os.path.join(HERE, "loss_golden.npz"), n=np.int64(len(CASES)), **out)


if __name__ == "__main__":
    ref_tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMGS_REFERENCE_TREE")
    if not ref_tree:
        sys.exit(f"usage: python {os.path.basename(__file__)} <reference tree> "
                 "(or set DMGS_REFERENCE_TREE)")
    main(ref_tree)
