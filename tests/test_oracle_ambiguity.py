"""The oracle's FP32-decidability band (oracle/raster.py, _blend_tile): a
pixel is flagged when a Gaussian's alpha lies within the FP32 reach of
1/255 — at least 1e-5 relative, more where the projected mean's pixel
coordinates are large (their float32 ulp) and the exponent is steep."""
import math

import torch

from oracle.raster import _blend_tile


def _one(x_mean, y_mean, conic, rel):
    """One Gaussian whose alpha at pixel (x_mean + dx, y_mean) is
    (1 + rel) / 255, with opacity 0.5."""
    a, b, c = conic
    op = 0.5
    # power = -a dx^2 / 2 must equal ln((1 + rel) / (255 op))
    power = math.log((1 + rel) / (255 * op))
    dx = math.sqrt(-2 * power / a)
    pix = torch.tensor([[x_mean + dx, y_mean]], dtype=torch.float64)
    xy = torch.tensor([[x_mean, y_mean]], dtype=torch.float64)
    co = torch.tensor([[a, b, c]], dtype=torch.float64)
    out, T, n, amb = _blend_tile(pix, xy, co, torch.tensor([op], dtype=torch.float64),
                                 torch.tensor([[1.0, 1.0, 1.0]], dtype=torch.float64),
                                 torch.zeros(3, dtype=torch.float64))
    return bool(amb[0]), int(n[0])


def test_fixed_band_near_the_origin():
    # small coordinates and a gentle exponent: the 1e-5 floor decides
    assert _one(10.0, 10.0, (0.01, 0.0, 0.01), 5e-6)[0]
    assert not _one(10.0, 10.0, (0.01, 0.0, 0.01), 5e-5)[0]


def test_mean_quantisation_widens_the_band():
    # at x = 1650 px a float32 coordinate is held to 1.2e-4 px; with a
    # steep exponent (d power / dx ~ 0.17) alpha moves ~2e-5 relative
    amb, n = _one(1650.2, 126.8, (0.0034, 0.0, 0.0048), 2e-5)
    assert amb and n == 1
    # the same relative offset near the origin is decidable
    assert not _one(10.2, 12.8, (0.0034, 0.0, 0.0048), 2e-5)[0]
    # and far enough from the threshold it is decidable at x = 1650 too
    assert not _one(1650.2, 126.8, (0.0034, 0.0, 0.0048), 1e-3)[0]
