"""Multi-view batched rendering: many views of one Gaussian set per launch.

The reference renders one view per call (``render_and_eval.py:42-44``,
``train_geo_stage2.py:101``).  Here a batch of up to 16 views of possibly
different resolutions is rendered forward and backward by one preprocess
pass (inputs read once), per-view binning into capacity-bounded lists, one
persistent blend launch over every view's tiles, and an adjoint that sums
the views' gradients (written once).  The calls never synchronise with the
host, so a whole step can be captured in a CUDA graph (:meth:`capture`).

:func:`autotune` picks the blend kernels' pixels-per-thread (1, 2, 4) and
Gaussians-per-batch (128, 256, 512) by timing.  (The binning tile stays
16 x 16: it defines which Gaussians reach which pixels, so another tile shape
would change the image relative to the reference.)
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time

import torch

from . import _lib
from ._lib import DmgsBatch, DmgsError, DmgsGaussians, DmgsGrads, DmgsView, check, ptr
from .rasterizer import GaussianRasterizationSettings, _f32, check_inputs

GAUSSIAN_KEYS = ("means3D", "opacities", "shs", "colors_precomp", "scales", "rotations",
                 "cov3D_precomp")

MAX_VIEWS = 16
# Blend tuning: (pixels per thread, Gaussians per staged batch, CTA shape);
# shape 0 = one 16x16 binning tile per CTA, 1 = 32x16 and 2 = 16x32 pixels
# (two adjacent binning tiles, each blended from its own list).
TILE_SHAPES = {0: "16x16", 1: "32x16", 2: "16x32"}
TUNE_SPACE = ([(p, b, 0) for p in (1, 2, 4) for b in (128, 256, 512)] +
              [(p, b, sh) for sh in (1, 2) for p in (2, 4) for b in (128, 256)])


def _view_struct(rs: GaussianRasterizationSettings, device, keep):
    bg = _f32(rs.bg, device)
    vm = _f32(rs.viewmatrix, device)
    pm = _f32(rs.projmatrix, device)
    cp = _f32(rs.campos, device)
    keep.extend([bg, vm, pm, cp])
    return DmgsView(int(rs.image_width), int(rs.image_height), float(rs.tanfovx),
                    float(rs.tanfovy), float(rs.scale_modifier), int(rs.sh_degree),
                    int(bool(rs.prefiltered)), int(bool(rs.debug)), ptr(bg), ptr(vm), ptr(pm),
                    ptr(cp))


class BatchedRasterizer:
    """Forward + backward of a fixed batch of views.

    ``gaussians``: dict of contiguous fp32 CUDA tensors with the reference's
    names (means3D, opacities, and shs or colors_precomp, and scales +
    rotations or cov3D_precomp).  Their storage is read at every call, so
    parameters updated in place are picked up (also by graph replays).

    ``means2D_grads``: keep each view's screen-space (NDC) mean gradient in
    ``self.means2D_grads[v]`` ([P, 3], the reference's
    ``viewspace_point_tensor.grad``).  ``densify_stats``: accumulate the
    reference's densification statistics (``add_densification_stats``,
    scene/gaussian_model.py:405-407) over every view of every backward into
    ``self.densify_accum`` / ``self.densify_count`` ([P] each; zeroed by
    :meth:`reset_densify_stats`) — the same information as the per-view
    gradients for training, without writing [P, 3] per view.
    """

    def __init__(self, settings, gaussians, capacity=None, margin=1.25, cfg=(4, 128, 0),
                 means2D_grads=True, densify_stats=False):
        if not 1 <= len(settings) <= MAX_VIEWS:
            raise ValueError(f"a batch holds 1..{MAX_VIEWS} views")
        check_inputs(**{k: gaussians.get(k) for k in GAUSSIAN_KEYS}, settings=settings)
        self.lib = _lib.load()
        self.settings = list(settings)
        self.g = {k: (None if v is None else _f32(v, v.device)) for k, v in gaussians.items()}
        self.device = self.g["means3D"].device
        self.P = self.g["means3D"].shape[0]
        self.M = self.g["shs"].shape[1] if self.g.get("shs") is not None else 0
        self.n = len(self.settings)
        if self.g.get("rotations") is not None and self.g["rotations"].data_ptr() % 16:
            self.g["rotations"] = self.g["rotations"].clone()
        self._keep = []
        self.views = (DmgsView * self.n)(*[_view_struct(s, self.device, self._keep)
                                           for s in self.settings])
        self.gauss = DmgsGaussians(self.P, self.M, ptr(self.g["means3D"]), ptr(self.g["opacities"]),
                                   ptr(self.g.get("shs")), ptr(self.g.get("colors_precomp")),
                                   ptr(self.g.get("scales")), ptr(self.g.get("rotations")),
                                   ptr(self.g.get("cov3D_precomp")))
        d = self.device
        self.images = [torch.empty(3, s.image_height, s.image_width, device=d) for s in self.settings]
        self.radii = [torch.empty(self.P, dtype=torch.int32, device=d) for _ in self.settings]
        self.dL_dout = [torch.zeros(3, s.image_height, s.image_width, device=d) for s in self.settings]
        self.grads = self._grad_buffers()
        self.means2D_grads = ([torch.empty(self.P, 3, device=d) for _ in self.settings]
                              if means2D_grads else None)
        self.densify_accum = torch.zeros(self.P, device=d) if densify_stats else None
        self.densify_count = torch.zeros(self.P, device=d) if densify_stats else None
        self.cfg = _cfg3(cfg)
        self.graph = None
        if capacity is None:
            capacity = [int(k * margin) + 1024 for k in self.count_instances()]
        self._set_capacity(capacity)

    # -- set-up ------------------------------------------------------------
    def _grad_buffers(self):
        d, P, g = self.device, self.P, self.g
        z = lambda *s: torch.empty(*s, device=d)  # noqa: E731
        return {"means3D": z(P, 3), "opacities": z(P, 1),
                "shs": z(P, self.M, 3) if g.get("shs") is not None else None,
                "colors_precomp": z(P, 3) if g.get("colors_precomp") is not None else None,
                "scales": z(P, 3) if g.get("scales") is not None and g.get("cov3D_precomp") is None else None,
                "rotations": z(P, 4) if g.get("rotations") is not None and g.get("cov3D_precomp") is None else None,
                "cov3D_precomp": z(P, 6) if g.get("cov3D_precomp") is not None else None}

    def count_instances(self):
        """Exact instance count of every view (one geometry pass per view;
        synchronises)."""
        lib, out = self.lib, []
        stream = _lib.stream_of(self.device)
        for v in range(self.n):
            s = self.settings[v]
            geom = torch.empty(lib.dmgs_geom_state_bytes(self.P, s.image_width, s.image_height),
                               dtype=torch.uint8, device=self.device)
            radii = torch.empty(max(self.P, 1), dtype=torch.int32, device=self.device)
            K = C.c_int64(0)
            check(lib.dmgs_raster_fwd_geometry(C.byref(self.views[v]), C.byref(self.gauss),
                                               geom.data_ptr(), geom.numel(), radii.data_ptr(),
                                               C.byref(K), stream), "batch count")
            out.append(int(K.value))
        return out

    def _set_capacity(self, capacity):
        self.capacity = [int(c) for c in capacity]
        self._cap = (C.c_int64 * self.n)(*self.capacity)
        self._out = (C.c_void_p * self.n)(*[t.data_ptr() for t in self.images])
        self._rad = (C.c_void_p * self.n)(*[t.data_ptr() for t in self.radii])
        self._dout = (C.c_void_p * self.n)(*[t.data_ptr() for t in self.dL_dout])
        self._m2 = ((C.c_void_p * self.n)(*[t.data_ptr() for t in self.means2D_grads])
                    if self.means2D_grads is not None else None)
        self.batch = DmgsBatch(self.n, self.views, self._out, self._rad, self._cap, *self.cfg)
        nbytes = self.lib.dmgs_batch_state_bytes(C.byref(self.batch), self.P)
        if nbytes == 0:
            raise DmgsError(-1, "batch", self.lib.dmgs_last_error().decode())
        self.state = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        g = self.grads
        self._grads = DmgsGrads(None, ptr(g["colors_precomp"]), ptr(g["opacities"]), ptr(g["means3D"]),
                                ptr(g["cov3D_precomp"]), ptr(g["shs"]), ptr(g["scales"]),
                                ptr(g["rotations"]))
        self.graph = None

    def set_config(self, ppt, batch, shape=0):
        """Blend tuning: pixels per thread, Gaussians per batch, CTA shape
        (see ``TILE_SHAPES``)."""
        self.cfg = _cfg3((ppt, batch, shape))
        self.batch.pixels_per_thread = self.cfg[0]
        self.batch.gaussians_per_batch = self.cfg[1]
        self.batch.tile_shape = self.cfg[2]
        self.graph = None

    # -- work ---------------------------------------------------------------
    def _enqueue_forward(self):
        check(self.lib.dmgs_raster_fwd_batched(C.byref(self.batch), C.byref(self.gauss),
                                               self.state.data_ptr(), self.state.numel(),
                                               _lib.stream_of(self.device)), "fwd_batched")

    def _enqueue_backward(self):
        check(self.lib.dmgs_raster_bwd_batched(C.byref(self.batch), C.byref(self.gauss), self._dout,
                                               self.state.data_ptr(), self.state.numel(),
                                               C.byref(self._grads), self._m2,
                                               ptr(self.densify_accum), ptr(self.densify_count),
                                               _lib.stream_of(self.device)), "bwd_batched")

    def reset_densify_stats(self):
        """Zero the densification accumulators (the reference re-creates
        them after each densification step)."""
        if self.densify_accum is not None:
            self.densify_accum.zero_()
            self.densify_count.zero_()

    def forward(self):
        """Render every view into ``self.images`` (asynchronous)."""
        self._enqueue_forward()
        return self.images

    def backward(self, dL_dimages=None):
        """Adjoint of the last forward; ``dL_dimages`` (optional list) is
        copied into the static gradient buffers first.  Gradients (summed
        over views) land in ``self.grads``."""
        if dL_dimages is not None:
            for dst, src in zip(self.dL_dout, dL_dimages):
                dst.copy_(src)
        self._enqueue_backward()
        return self.grads

    def step(self):
        """Forward + backward with the current ``dL_dout`` buffers; replays
        the captured graph when there is one."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._enqueue_forward()
            self._enqueue_backward()

    def capture(self):
        """Capture forward + backward in a CUDA graph (replayed by step())."""
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):  # warm the kernels' one-time attribute set-up
            self._enqueue_forward()
            self._enqueue_backward()
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._enqueue_forward()
            self._enqueue_backward()
        self.graph = g
        return g

    def status(self):
        """Per-view instance counts; raises DmgsError on capacity overflow
        (grow with :meth:`grow`)."""
        K = (C.c_int64 * self.n)()
        code = self.lib.dmgs_batch_status(C.byref(self.batch), self.P, self.state.data_ptr(),
                                          self.state.numel(), K, _lib.stream_of(self.device))
        counts = [int(k) for k in K]
        check(code, "batch_status")
        return counts

    def counters(self):
        """Per-view binning counters of the last forward (synchronises): a
        dict per view with the instances K, the row-list entries K1, the
        visible Gaussians V, the chunks C and the longest tile list."""
        words = (C.c_uint32 * (16 * self.n))()
        check(self.lib.dmgs_batch_counters(C.byref(self.batch), self.P, self.state.data_ptr(),
                                           self.state.numel(), words, _lib.stream_of(self.device)),
              "batch_counters")
        return [{"K": words[16 * v + 1], "K1": words[16 * v + 2], "maxlist": words[16 * v + 3],
                 "V": words[16 * v + 4], "C": words[16 * v + 8]} for v in range(self.n)]

    def grow(self, factor=1.5):
        """Re-plan capacities from exact counts (after an overflow)."""
        self._set_capacity([int(k * factor) + 1024 for k in self.count_instances()])


class HostPipeline:
    """Training steps whose inputs come from host memory and whose results go
    back to it, overlapped: while step i computes, the upload of step i+1 and
    the download of step i-1 run on their own copy streams.  Two
    BatchedRasterizers (ping-pong device buffers, each replaying its own CUDA
    graph) hold the Gaussians, image gradients and outputs of alternate steps.

    ``names``: the Gaussian tensors uploaded every step (keys of
    ``gaussians``); the rasteriser options (capacity, cfg, means2D_grads,
    densify_stats) pass through ``**kw``."""

    def __init__(self, settings, gaussians, names, **kw):
        self.names = list(names)
        self.slots = [BatchedRasterizer(settings, {k: v.detach().clone() for k, v in
                                                   gaussians.items() if v is not None}, **kw)
                      for _ in range(2)]
        for br in self.slots:
            br.capture()
        dev = self.slots[0].device
        self.up = torch.cuda.Stream(device=dev)
        self.comp = torch.cuda.Stream(device=dev)
        self.down = torch.cuda.Stream(device=dev)
        # Per slot: its last compute done (its inputs may be overwritten) and
        # its last download done (its outputs may be overwritten).  An upload
        # waits only for the former, a compute for the latter, so neither
        # copy direction waits for the other.
        self.inputs_free = [None, None]
        self.outputs_free = [None, None]
        self.last = None
        self.i = 0

    def set_config(self, ppt, batch, shape=0):
        for br in self.slots:
            br.set_config(ppt, batch, shape)
            br.capture()

    def start(self):
        """Order the pipeline after the work already on the current stream."""
        cur = torch.cuda.current_stream(self.slots[0].device)
        for st in (self.up, self.comp, self.down):
            st.wait_stream(cur)

    def submit(self, host_gaussians, host_dout, host_images, host_grads):
        """Enqueue one step: upload host_gaussians (dict) and host_dout (list
        of [3,H,W]), forward + backward, download the images into
        host_images and the gradients named in ``names`` into host_grads.
        Host buffers must be pinned and stay untouched until the returned
        event has completed."""
        k = self.i % 2
        self.i += 1
        br = self.slots[k]
        if self.inputs_free[k] is not None:
            self.up.wait_event(self.inputs_free[k])
        with torch.cuda.stream(self.up):
            for n in self.names:
                br.g[n].copy_(host_gaussians[n], non_blocking=True)
            for d, h in zip(br.dL_dout, host_dout):
                d.copy_(h, non_blocking=True)
            uploaded = torch.cuda.Event()
            uploaded.record(self.up)
        self.comp.wait_event(uploaded)
        if self.outputs_free[k] is not None:
            self.comp.wait_event(self.outputs_free[k])
        with torch.cuda.stream(self.comp):
            br.graph.replay()
            computed = torch.cuda.Event()
            computed.record(self.comp)
        self.down.wait_event(computed)
        with torch.cuda.stream(self.down):
            for h, d in zip(host_images, br.images):
                h.copy_(d, non_blocking=True)
            for n in self.names:
                host_grads[n].copy_(br.grads[n], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.down)
        self.inputs_free[k] = computed
        self.outputs_free[k] = done
        self.last = done
        return done

    def finish(self):
        """Make the current stream wait for every submitted step."""
        cur = torch.cuda.current_stream(self.slots[0].device)
        for st in (self.up, self.comp, self.down):
            cur.wait_stream(st)


def _cfg3(cfg):
    """(pixels per thread, batch[, shape]) -> a 3-tuple of ints (shape 0 if absent)."""
    c = tuple(int(x) for x in cfg)
    return c if len(c) == 3 else (c[0], c[1], 0)


def config_name(cfg):
    ppt, b, sh = _cfg3(cfg)
    return f"{ppt}x{b}@{TILE_SHAPES[sh]}"


def autotune(br: BatchedRasterizer, space=TUNE_SPACE, iters=5, cache_path=None):
    """Time forward + backward for every (pixels/thread, batch, CTA shape)
    in ``space`` and keep the fastest; the choice is cached in JSON at
    ``cache_path`` (default ``$DMGS_AUTOTUNE_CACHE`` if set) keyed by device,
    P and resolutions."""
    key = json.dumps([torch.cuda.get_device_name(br.device), br.P,
                      [(s.image_width, s.image_height) for s in br.settings]])
    cache_path = cache_path or os.environ.get("DMGS_AUTOTUNE_CACHE")
    cache = {}
    if cache_path and os.path.exists(cache_path):
        try:
            cache = json.load(open(cache_path))
        except Exception:
            cache = {}
    if key in cache:
        br.set_config(*cache[key]["best"])
        return cache[key]
    times, names = {}, {}
    for cfg in space:
        br.set_config(*cfg)
        br.step()
        torch.cuda.synchronize(br.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(iters):
            br.step()
        e1.record()
        torch.cuda.synchronize(br.device)
        name = config_name(cfg)
        times[name] = e0.elapsed_time(e1) / iters
        names[name] = _cfg3(cfg)
    best = min(times, key=times.get)
    br.set_config(*names[best])
    result = {"best": list(names[best]), "ms": times, "when": time.time(),
              "axes": {"pixels_per_thread": sorted({c[0] for c in names.values()}),
                       "gaussians_per_batch": sorted({c[1] for c in names.values()}),
                       "cta_shape": [TILE_SHAPES[k] for k in sorted({c[2] for c in names.values()})]}}
    if cache_path:
        cache[key] = result
        os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        json.dump(cache, open(cache_path, "w"), indent=1)
    return result


class _RasterizeBatched(torch.autograd.Function):
    @staticmethod
    def forward(ctx, br, means3D, opacities, shs, colors, scales, rotations, cov3D):
        br.forward()
        ctx.br = br
        return tuple(img.clone() for img in br.images)

    @staticmethod
    def backward(ctx, *dimgs):
        br = ctx.br
        br.backward([d if d is not None else torch.zeros_like(i) for d, i in zip(dimgs, br.images)])
        g = br.grads
        return (None, g["means3D"].clone(), g["opacities"].clone(),
                None if g["shs"] is None else g["shs"].clone(),
                None if g["colors_precomp"] is None else g["colors_precomp"].clone(),
                None if g["scales"] is None else g["scales"].clone(),
                None if g["rotations"] is None else g["rotations"].clone(),
                None if g["cov3D_precomp"] is None else g["cov3D_precomp"].clone())


def rasterize_batched(br: BatchedRasterizer, means3D, opacities, shs=None, colors_precomp=None,
                      scales=None, rotations=None, cov3D_precomp=None):
    """Autograd entry: images of every view of ``br``; the inputs must be the
    tensors ``br`` was built on (their gradients are the sums over views)."""
    return _RasterizeBatched.apply(br, means3D, opacities, shs, colors_precomp, scales, rotations,
                                   cov3D_precomp)
