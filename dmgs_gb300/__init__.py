"""dmgs_gb300 — GB300 (sm_103a) rasteriser and face binding of DMGS's hot path.

Public surface:

* :mod:`dmgs_gb300.rasterizer` — drop-in for the ``diff_gaussian_rasterization``
  module the reference imports (``GaussianRasterizationSettings``,
  ``GaussianRasterizer``, ``rasterize_gaussians``);
* :mod:`dmgs_gb300.binding` — fused mesh -> Gaussian binding
  (stage-2 covariance form and stage-3 scale/rotation form) with adjoints;
* :func:`install_as_diff_gaussian_rasterization` — registers the drop-in
  under the reference's module name so ``gaussian_renderer`` runs unchanged.
"""
from __future__ import annotations

import sys

from .rasterizer import (GaussianRasterizationSettings, GaussianRasterizer,  # noqa: F401
                         rasterize_gaussians)

__all__ = ["GaussianRasterizationSettings", "GaussianRasterizer", "rasterize_gaussians",
           "install_as_diff_gaussian_rasterization"]


def install_as_diff_gaussian_rasterization():
    """Make ``import diff_gaussian_rasterization`` resolve to this package's
    rasteriser (call before importing the reference's ``gaussian_renderer``)."""
    from . import rasterizer
    sys.modules["diff_gaussian_rasterization"] = rasterizer
    return rasterizer
