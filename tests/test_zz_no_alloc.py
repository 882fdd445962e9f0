"""The allocation-free backward entry point, dmgs_raster_bwd_noalloc.

It serves callers that cannot allocate device memory (a plugin inside an
application that owns the GPU's memory pool, a real-time loop that must not
call cudaMalloc between frames): its scratch is a static device array of
the library.  This test calls it through the C ABI twice in a row — the
second call reuses the array the first one filled — and checks both results
against dmgs_raster_bwd with a caller-provided scratch buffer.  It also
checks that a scene above the static limit is refused with a clear error.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from dmgs_gb300 import _lib
from dmgs_gb300._lib import DmgsError, DmgsGaussians, DmgsGrads, ptr
from dmgs_gb300.scenes import small_scene
from helpers import AbiRun, mode_inputs, rel_l2

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-3  # relative L2, the tolerance of the other gradient tests


def _grad_buffers(run):
    P, M, d = run.P, run.M, run.device
    z = lambda *s: torch.full(s, float("nan"), device=d)  # noqa: E731  (must be fully written)
    gr = dict(means2D=z(P, 3), colors=z(P, 3), opacities=z(P, 1), means3D=z(P, 3),
              shs=z(P, M, 3), scales=z(P, 3), rotations=z(P, 4))
    desc = DmgsGrads(ptr(gr["means2D"]), ptr(gr["colors"]), ptr(gr["opacities"]),
                     ptr(gr["means3D"]), None, ptr(gr["shs"]), ptr(gr["scales"]),
                     ptr(gr["rotations"]))
    return gr, desc


def _noalloc_backward(run, dout):
    lib = _lib.load()
    gr, desc = _grad_buffers(run)
    _lib.check(lib.dmgs_raster_bwd_noalloc(run.view, run.g, dout.data_ptr(), run.geom.data_ptr(),
                                           run.geom.numel(), run.bin.data_ptr(), run.bin.numel(),
                                           run.K, run.img.data_ptr(), run.img.numel(), desc,
                                           run.stream), "raster_bwd_noalloc")
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in gr.items()}


def test_noalloc_backward_matches_allocating_entry_point():
    sc = small_scene(P=6000, width=160, height=128, seed=31)
    run = AbiRun(sc.views[0], mode_inputs(sc, ("shs", "sr")), debug=False).forward()
    dimg = np.random.default_rng(31).standard_normal((3, 128, 160)).astype(np.float32)
    ref = run.backward(dimg)  # dmgs_raster_bwd with a torch-allocated scratch buffer
    dout = torch.tensor(dimg, device="cuda")
    for call in range(2):
        got = _noalloc_backward(run, dout)
        for name, v in got.items():
            assert np.isfinite(v).all(), (call, name)
            assert rel_l2(v, ref[name]) <= GRAD_TOL, (call, name, rel_l2(v, ref[name]))


def test_noalloc_backward_refuses_scenes_above_the_limit():
    lib = _lib.load()
    limit = 262144
    sc = small_scene(P=16, width=32, height=32, seed=32)
    run = AbiRun(sc.views[0], mode_inputs(sc, ("shs", "sr")), debug=False).forward()
    t = run.t
    big = DmgsGaussians(limit + 1, run.M, ptr(t["means3D"]), ptr(t["opacities"]), ptr(t["shs"]),
                        None, ptr(t["scales"]), ptr(t["rotations"]), None)
    _, desc = _grad_buffers(run)
    dout = torch.zeros(3, 32, 32, device="cuda")
    code = lib.dmgs_raster_bwd_noalloc(run.view, big, dout.data_ptr(), run.geom.data_ptr(),
                                       run.geom.numel(), run.bin.data_ptr(), run.bin.numel(), run.K,
                                       run.img.data_ptr(), run.img.numel(), desc, run.stream)
    assert code == -1
    assert b"static scratch limit" in lib.dmgs_last_error()
    with pytest.raises(DmgsError):
        _lib.check(code, "raster_bwd_noalloc")
