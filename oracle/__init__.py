"""CPU oracle for the DMGS hot path — TEST INFRASTRUCTURE ONLY.

Nothing in the product path (``dmgs_gb300``) imports this package.  It is
imported only by ``tests/``, by ``__graft_entry__.smoke()`` (to check the CUDA path's result)
and by ``bench.py``'s CPU baseline / ``--impl reference`` leg.

Modules
-------
raster   Gaussian rasteriser: FP32 emulation of the integer-determining
         geometry stage (bit-exact radii, tile rectangles, depth keys,
         sorted tile lists and ranges) and an FP64 torch restatement of
         the blending forward pass whose autograd backward reproduces the
         reference adjoint's conventions.
binding  Mesh -> Gaussian face binding (stage-2 covariance form and the
         stage-3 scale/rotation form), FP64 torch restatement.
flexicubes  FlexiCubes triangle extraction on a regular grid (both
         quad-splitting modes) and, by autograd, its adjoint; float64 by
         default, float32 on request.
texture  The hash-grid texture (multiresolution hash encoding + bias-free
         MLP, ``MLPTexture3D.sample_noact``) and its adjoint.

Parity status
-------------
* Rasteriser core: PARITY UNPINNED.  The reference's rasteriser is the
  un-vendored git submodule ``submodules/diff-gaussian-rasterization``
  (``.gitmodules:4-6``, graphdeco-inria/diff-gaussian-rasterization at an
  unknown commit); no source, tests or golden vectors for it exist in the
  reference tree.  The oracle restates the published 3DGS / EWA-splatting
  algorithm.  Its conventions that DO live in the reference tree are pinned
  by golden vectors generated from the reference's own Python
  (``tests/golden/make_golden.py``): SH evaluation
  (``utils/sh_utils.py:25-110``), quaternion -> rotation and covariance
  packing (``utils/general_utils.py:64-110``), camera matrices
  (``utils/graphics_utils.py:38-71``, ``scene/cameras.py:54-57``).
* Binding: pinned against the reference's own ``renew_gaussian`` /
  ``get_covariance_dyn`` (``scene/gaussian_geo_model_mlp_flex.py:258-385``)
  run on CPU in the build container (fixtures in ``tests/golden/``).
* FlexiCubes: pinned against the reference's own class
  (``geo/flexicubes.py``) run on the CPU (``tests/golden/flexicubes_golden.npz``)
  and its tables against ``geo/tables.py``.
* Texture: the code around the encoding is pinned against the reference's
  ``MLPTexture3D`` (``tests/golden/texture_golden.npz``); the encoding itself
  lives in the absent third-party tiny-cuda-nn: ENCODING PARITY UNPINNED
  (restated from the published algorithm).
"""
