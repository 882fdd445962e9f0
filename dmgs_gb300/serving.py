"""Serving loop: continuous batching of render requests for resident scenes.

The reference has no serving path (it renders one view per call,
``render_and_eval.py:42-44``).  Here several scenes stay resident on the
device and render requests (scene, camera, resolution) arrive over time.
The scheduler keeps a FIFO of arrived requests and, whenever a slot and
enough of the HBM budget are free, admits the next ones into a *wave*: one
``dmgs_render_multi`` launch sequence renders every request of the wave
(each with its own scene) — per-request preprocess and capacity-bounded
binning, then one persistent blend over all the wave's tiles.  Waves go to
several CUDA streams in turn, so a wave admitted while others run overlaps
with them on the device.  Completion is observed through events; a request
whose instance list overflowed its capacity is re-admitted at the head of
the queue with the exact count the device reported.  Memory is accounted per
request (its state bytes plus its image), released when its wave completes.

Cancellation and timeouts are host decisions (no kernel is interrupted): a
request cancelled, or not admitted within its ``admit_timeout`` seconds of
arriving, leaves the queue unrendered; one cancelled while its wave runs is
rendered with the wave but its result is dropped (neither delivered nor
re-admitted after an overflow).  Each request ends with ``status`` "done",
"cancelled" or "timeout".

The scheduler is independent of the device: :class:`Scheduler` drives a
backend (``footprint``/``reserve``/``launch``/``ready``/``results``/
``release``), so its admission, ordering and retry logic is tested on the CPU
with a fake one.  The GPU backend places every admitted request's state and
image in one device arena allocated up front (first fit, coalescing frees),
so serving does no device allocation.
"""
from __future__ import annotations

import ctypes as C
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

ST_OVERFLOW = 2
ST_ERRORS = 1 | 4  # prefiltered point culled, index out of its buffer


@dataclass
class Request:
    rid: int
    scene: int
    view: object          # camera.ViewSpec
    arrival: float        # seconds after the start of the run
    capacity: int = 0     # instance-list capacity of the current attempt
    attempts: int = 0
    t_admit: float = -1.0
    t_done: float = -1.0
    result: object = None  # the image (host copy when the backend copies out)
    blocks: object = None  # backend placement while admitted
    admit_timeout: float | None = None  # seconds after arrival to be admitted by, or dropped
    cancelled: bool = False  # set by the client (any thread); see Scheduler.cancel
    status: str = ""       # "done", "cancelled" or "timeout" once finished

    @property
    def key(self):
        return (self.scene, self.view.width, self.view.height)

    @property
    def latency(self):
        return self.t_done - self.arrival


class CapacityEstimator:
    """Instance-list capacity per (scene, width, height): the largest count
    seen times `margin`, plus `slack`; `default(req)` before any
    observation."""

    def __init__(self, margin=1.3, slack=4096, default=None):
        self.margin, self.slack = margin, slack
        self.seen = {}
        self.default = default or (lambda req: 1 << 20)

    def observe(self, req, K):
        self.seen[req.key] = max(self.seen.get(req.key, 0), int(K))

    def capacity(self, req):
        k = self.seen.get(req.key)
        if k is None:
            return int(self.default(req))
        return int(k * self.margin) + self.slack


@dataclass
class Wave:
    reqs: list
    nbytes: int
    handle: object
    stream: int


@dataclass
class ServeStats:
    latencies_ms: list = field(default_factory=list)
    waves: int = 0
    retries: int = 0
    cancelled: int = 0
    timeouts: int = 0
    peak_bytes: int = 0
    peak_inflight: int = 0
    wall_s: float = 0.0

    def summary(self):
        lat = np.asarray(self.latencies_ms)
        n = len(lat)
        return {"requests": n,
                "p50_ms": float(np.percentile(lat, 50)) if n else None,
                "p99_ms": float(np.percentile(lat, 99)) if n else None,
                "mean_ms": float(lat.mean()) if n else None,
                "max_ms": float(lat.max()) if n else None,
                "views_per_s": n / self.wall_s if self.wall_s > 0 else None,
                "waves": self.waves, "mean_wave": n / self.waves if self.waves else None,
                "retries": self.retries, "cancelled": self.cancelled,
                "timeouts": self.timeouts, "peak_bytes": self.peak_bytes,
                "peak_inflight": self.peak_inflight, "wall_s": self.wall_s}


class Scheduler:
    """Admission and continuous batching over a backend.

    budget_bytes: HBM the in-flight requests may hold; max_inflight: request
    slots; max_wave: requests per launch (<= 16); n_streams: waves in flight
    rotate over this many streams.  `clock()` returns seconds; `idle()` is
    called when there is nothing to do (the real loop sleeps briefly)."""

    def __init__(self, backend, budget_bytes, max_inflight=64, max_wave=16, n_streams=None,
                 estimator=None, clock=time.perf_counter, idle=None):
        if not 1 <= max_wave <= 16:
            raise ValueError("a wave holds 1..16 requests")
        self.backend = backend
        self.budget = int(budget_bytes)
        self.max_inflight = max_inflight
        self.max_wave = max_wave
        self.n_streams = n_streams or getattr(backend, "n_streams", 4)
        self.estimator = estimator or CapacityEstimator()
        self.clock = clock
        self.idle = idle or (lambda: time.sleep(50e-6))
        self._cancel_posted = False

    def cancel(self, request):
        """Cancel a request (callable from another thread or from `deliver`):
        it is dropped from the queue, or its result is dropped if its wave is
        already running."""
        request.cancelled = True
        self._cancel_posted = True

    @staticmethod
    def _dropped(r, now, st):
        """Whether queued request r leaves unrendered now (cancelled, or not
        admitted within its timeout; a retry after an overflow keeps its
        place); marks it."""
        if r.cancelled:
            r.status, st.cancelled = "cancelled", st.cancelled + 1
        elif r.admit_timeout is not None and r.attempts == 0 and now - r.arrival > r.admit_timeout:
            r.status, st.timeouts = "timeout", st.timeouts + 1
        else:
            return False
        r.t_done, r.result = now, None
        return True

    def run(self, requests, deliver=None):
        """Serve `requests` (arrival times in seconds from the start) in real
        time; returns ServeStats.  Each request gets t_admit, t_done, status
        and result; `deliver(request)`, if given, is called as each completes
        (a client taking the image; it may recycle the buffer).  Cancelled
        and timed-out requests are not delivered."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        be, est = self.backend, self.estimator
        pending, inflight = deque(), []
        st = ServeStats()
        used = n_in = done = nxt = 0
        stream = 0
        # the queue is scanned for drops only when some request can be dropped
        timeouts = any(r.admit_timeout is not None for r in reqs)
        self._cancel_posted = self._cancel_posted or any(r.cancelled for r in reqs)
        t0 = self.clock()
        while done < len(reqs):
            now = self.clock() - t0
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                pending.append(reqs[nxt])
                nxt += 1
            if pending and (timeouts or self._cancel_posted):
                self._cancel_posted = False
                keep = deque()
                for r in pending:
                    if self._dropped(r, now, st):
                        done += 1
                    else:
                        keep.append(r)
                pending = keep
            progressed = False
            for w in list(inflight):
                if not be.ready(w.handle):
                    continue
                progressed = True
                t_obs = self.clock() - t0
                retry = []
                for r, (status, K) in zip(w.reqs, be.results(w.handle)):
                    est.observe(r, K)
                    if status & ST_ERRORS:
                        raise RuntimeError(f"request {r.rid}: device status {status}")
                    if r.cancelled:  # rendered, but nobody wants it any more
                        if r.result is not None and hasattr(be, "recycle"):
                            be.recycle(r)  # its host buffer back to the backend's pool
                        r.status, r.t_done, r.result = "cancelled", t_obs, None
                        st.cancelled += 1
                        done += 1
                    elif status & ST_OVERFLOW:
                        r.capacity = int(K) + est.slack
                        r.result = None
                        retry.append(r)
                        st.retries += 1
                    else:
                        r.t_done, r.status = t_obs, "done"
                        st.latencies_ms.append(1e3 * r.latency)
                        done += 1
                        if deliver is not None:
                            deliver(r)
                for r in reversed(retry):  # back at the head of the queue, in order
                    pending.appendleft(r)
                be.release(w.handle)
                used -= w.nbytes
                n_in -= len(w.reqs)
                inflight.remove(w)
            wave, wbytes = [], 0
            while pending and len(wave) < self.max_wave and n_in + len(wave) < self.max_inflight:
                r = pending[0]
                if self._dropped(r, now, st):  # cancelled after the last scan
                    pending.popleft()
                    done += 1
                    continue
                cap = r.capacity or est.capacity(r)
                fb = be.footprint(r, cap)
                if fb > self.budget:
                    raise RuntimeError(f"request {r.rid} needs {fb} bytes, above the budget")
                if used + wbytes + fb > self.budget:
                    break
                if not be.reserve(r, cap):  # the backend could not place it (fragmentation)
                    if n_in == 0 and not wave:
                        raise RuntimeError(f"request {r.rid} cannot be placed in the backend's memory")
                    break
                pending.popleft()
                r.capacity = cap
                r.attempts += 1
                r.t_admit = self.clock() - t0
                wave.append(r)
                wbytes += fb
            if wave:
                handle = be.launch(wave, [r.capacity for r in wave], stream)
                inflight.append(Wave(wave, wbytes, handle, stream))
                stream = (stream + 1) % self.n_streams
                used += wbytes
                n_in += len(wave)
                st.waves += 1
                st.peak_bytes = max(st.peak_bytes, used)
                st.peak_inflight = max(st.peak_inflight, n_in)
                progressed = True
            if not progressed:
                self.idle()
        st.wall_s = max(r.t_done for r in reqs) - min(r.arrival for r in reqs) if reqs else 0.0
        return st


def poisson_trace(rate, seconds, n_scenes, resolutions, seed=0, view_fn=None):
    """Requests with Poisson arrivals at `rate` per second for `seconds`,
    scene uniform over n_scenes, resolution uniform over `resolutions`,
    camera from view_fn(rng, width, height)."""
    from .scenes import random_inside_view
    view_fn = view_fn or random_inside_view
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        w, h = resolutions[rng.integers(len(resolutions))]
        out.append(Request(len(out), int(rng.integers(n_scenes)), view_fn(rng, w, h), t))
    return out


# --------------------------------------------------------------------------
# GPU backends
# --------------------------------------------------------------------------

class _PinnedPool:
    """Reusable page-locked host buffers by element count."""

    def __init__(self, torch, dtype):
        self.torch, self.dtype, self.free = torch, dtype, {}

    def get(self, n):
        lst = self.free.get(n)
        if lst:
            return lst.pop()
        return self.torch.empty(n, dtype=self.dtype, pin_memory=True)

    def put(self, buf):
        self.free.setdefault(buf.numel(), []).append(buf)


class DeviceArena:
    """One device buffer carved into 256-byte-aligned blocks: first fit over
    an offset-sorted free list, neighbours coalesced on release."""

    ALIGN = 256

    def __init__(self, nbytes, device):
        import torch
        self.size = int(nbytes) // self.ALIGN * self.ALIGN
        self.buf = torch.empty(self.size, dtype=torch.uint8, device=device)
        self.base = self.buf.data_ptr()
        self.free = [(0, self.size)]
        self.used = 0

    def _round(self, n):
        return (int(n) + self.ALIGN - 1) // self.ALIGN * self.ALIGN

    def alloc(self, n):
        n = self._round(max(int(n), 1))
        for i, (o, sz) in enumerate(self.free):
            if sz >= n:
                if sz == n:
                    del self.free[i]
                else:
                    self.free[i] = (o + n, sz - n)
                self.used += n
                return o
        return None

    def release(self, o, n):
        import bisect
        n = self._round(max(int(n), 1))
        self.used -= n
        i = bisect.bisect_left(self.free, (o, 0))
        self.free.insert(i, (o, n))
        if i + 1 < len(self.free) and o + n == self.free[i + 1][0]:  # merge right
            self.free[i] = (o, n + self.free[i + 1][1])
            del self.free[i + 1]
        if i > 0 and self.free[i - 1][0] + self.free[i - 1][1] == o:  # merge left
            self.free[i - 1] = (self.free[i - 1][0], self.free[i - 1][1] + self.free[i][1])
            del self.free[i]

    def tensor(self, o, n, dtype, shape):
        import torch
        esz = torch.tensor([], dtype=dtype).element_size()
        return self.buf[o:o + n * esz].view(dtype).view(*shape)


class ResidentScene:
    """A scene kept on the device: the reference's tensors (means3D,
    opacities, shs, scales, rotations) and the C-ABI view of them."""

    def __init__(self, tensors, sh_degree=3):
        from . import _lib
        from .rasterizer import check_inputs
        check_inputs(tensors.get("means3D"), tensors.get("opacities"), tensors.get("shs"),
                     scales=tensors.get("scales"), rotations=tensors.get("rotations"))
        self.t = {k: v.contiguous().float() for k, v in tensors.items()}
        self.P = self.t["means3D"].shape[0]
        self.M = self.t["shs"].shape[1]
        self.sh_degree = sh_degree
        p = _lib.ptr
        self.gauss = _lib.DmgsGaussians(self.P, self.M, p(self.t["means3D"]), p(self.t["opacities"]),
                                        p(self.t["shs"]), None, p(self.t["scales"]),
                                        p(self.t["rotations"]), None)
        self.nbytes = sum(v.numel() * v.element_size() for v in self.t.values())


class GpuBackend:
    """Waves rendered by dmgs_render_multi on a set of streams.  Each
    admitted request holds two arena blocks (its state and its image) from
    reserve() until its wave is released; camera constants go up in one copy
    per wave, status words (and, with copy_out, the images) come back into
    pinned host memory."""

    CAM = 16 + 16 + 3 + 3  # view matrix, full projection, campos, background

    def __init__(self, scenes, arena_bytes=8 << 30, n_streams=4, cfg=(4, 128), copy_out=True,
                 device=None, max_waves=256):
        import torch
        from . import _lib
        self.torch, self._lib = torch, _lib
        self.lib = _lib.load()
        self.scenes = scenes
        self.device = device or torch.device("cuda")
        self.arena = DeviceArena(arena_bytes, self.device)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(n_streams)]
        self.n_streams = n_streams
        self.cfg = cfg
        self.copy_out = copy_out
        self.f32 = _PinnedPool(torch, torch.float32)
        self.u32 = _PinnedPool(torch, torch.int32)
        self.queues = torch.zeros(max_waves * 64, dtype=torch.int32, device=self.device)
        self.free_queues = list(range(max_waves))
        self._sb_cache = {}

    def _view(self, r, cam_ptr):
        v = r.view
        return self._lib.DmgsView(v.width, v.height, float(v.tanfovx), float(v.tanfovy), 1.0,
                                  self.scenes[r.scene].sh_degree, 0, 0, cam_ptr + 4 * 35, cam_ptr,
                                  cam_ptr + 4 * 16, cam_ptr + 4 * 32)

    def _state_bytes(self, r, cap):
        key = (r.scene, r.view.width, r.view.height, int(cap))
        sb = self._sb_cache.get(key)
        if sb is None:
            view = self._view(r, 0)
            sb = int(self.lib.dmgs_multi_view_state_bytes(C.byref(view),
                                                          C.byref(self.scenes[r.scene].gauss),
                                                          int(cap)))
            self._sb_cache[key] = sb
        return sb

    def footprint(self, r, cap):
        return self.arena._round(self._state_bytes(r, cap)) + self.arena._round(
            12 * r.view.width * r.view.height)

    def reserve(self, r, cap):
        sb = self._state_bytes(r, cap)
        ib = 12 * r.view.width * r.view.height
        o1 = self.arena.alloc(sb)
        if o1 is None:
            return False
        o2 = self.arena.alloc(ib)
        if o2 is None:
            self.arena.release(o1, sb)
            return False
        r.blocks = (o1, sb, o2, ib)
        return True

    def launch(self, reqs, caps, stream):
        torch, L = self.torch, self._lib
        s = self.streams[stream % len(self.streams)]
        n = len(reqs)
        cam_host = self.f32.get(n * self.CAM)
        ch = cam_host.numpy().reshape(n, self.CAM)
        for i, r in enumerate(reqs):
            v = r.view
            ch[i, 0:16] = np.asarray(v.viewmatrix, np.float32).reshape(16)
            ch[i, 16:32] = np.asarray(v.projmatrix, np.float32).reshape(16)
            ch[i, 32:35] = v.campos
            ch[i, 35:38] = 0.0
        status = self.u32.get(2 * n)
        q = self.free_queues.pop()
        ar = self.arena
        with torch.cuda.stream(s):
            cam_dev = torch.empty(n * self.CAM, device=self.device)
            cam_dev.copy_(cam_host, non_blocking=True)
            base = cam_dev.data_ptr()
            views = (L.DmgsView * n)(*[self._view(r, base + 4 * i * self.CAM)
                                       for i, r in enumerate(reqs)])
            images = [ar.tensor(r.blocks[2], 3 * r.view.width * r.view.height, torch.float32,
                                (3, r.view.height, r.view.width)) for r in reqs]
            out = (C.c_void_p * n)(*[im.data_ptr() for im in images])
            states = (C.c_void_p * n)(*[ar.base + r.blocks[0] for r in reqs])
            sizes = (C.c_size_t * n)(*[r.blocks[1] for r in reqs])
            capa = (C.c_int64 * n)(*caps)
            gauss = (L.DmgsGaussians * n)(*[self.scenes[r.scene].gauss for r in reqs])
            b = L.DmgsBatch(n, views, out, None, capa, *self.cfg)
            queue = self.queues.data_ptr() + 256 * q
            L.check(self.lib.dmgs_render_multi(C.byref(b), gauss, states, sizes, queue,
                                               s.cuda_stream), "render_multi")
            L.check(self.lib.dmgs_multi_status_async(C.byref(b), gauss, states, sizes,
                                                     status.data_ptr(), s.cuda_stream),
                    "multi_status")
            host_imgs = None
            if self.copy_out:
                host_imgs = [self.f32.get(im.numel()) for im in images]
                for h, im in zip(host_imgs, images):
                    h.copy_(im.view(-1), non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(s)
        return {"ev": ev, "status": status, "cam": cam_host, "cam_dev": cam_dev, "q": q,
                "images": images, "host": host_imgs, "reqs": reqs}

    def ready(self, h):
        return h["ev"].query()

    def results(self, h):
        s = h["status"].numpy()
        out = []
        for i, r in enumerate(h["reqs"]):
            out.append((int(s[2 * i]) & 0xffffffff, int(s[2 * i + 1]) & 0xffffffff))
            if self.copy_out:
                r.result = h["host"][i].view(3, r.view.height, r.view.width)
            else:
                r.result = h["images"][i].clone()
        return out

    def release(self, h):
        for r in h["reqs"]:
            o1, sb, o2, ib = r.blocks
            self.arena.release(o1, sb)
            self.arena.release(o2, ib)
            r.blocks = None
        self.f32.put(h["cam"])
        self.u32.put(h["status"])
        self.free_queues.append(h["q"])
        h.clear()

    def recycle(self, req):
        """Return a delivered request's pinned result buffer to the pool."""
        if self.copy_out and req.result is not None:
            self.f32.put(req.result.view(-1))
            req.result = None


class PlainBackend:
    """One request at a time through the drop-in rasteriser (the reference's
    call pattern: GaussianRasterizer forward per view, host-synchronising
    on its instance count), with the same result copy as GpuBackend."""

    def __init__(self, scenes, copy_out=True, device=None):
        import torch
        self.torch = torch
        self.scenes = scenes
        self.device = device or torch.device("cuda")
        self.copy_out = copy_out
        self.f32 = _PinnedPool(torch, torch.float32)

    def footprint(self, req, cap):
        return 1

    def reserve(self, req, cap):
        return True

    def launch(self, reqs, caps, stream):
        import torch
        from .rasterizer import GaussianRasterizationSettings, GaussianRasterizer
        r = reqs[0]
        sc, v = self.scenes[r.scene], r.view
        t = lambda a: torch.as_tensor(np.asarray(a, np.float32)).to(self.device, non_blocking=True)  # noqa: E731
        rs = GaussianRasterizationSettings(
            image_height=v.height, image_width=v.width, tanfovx=v.tanfovx,
            tanfovy=v.tanfovy, bg=torch.zeros(3, device=self.device),
            scale_modifier=1.0, viewmatrix=t(v.viewmatrix), projmatrix=t(v.projmatrix),
            sh_degree=sc.sh_degree, campos=t(v.campos), prefiltered=False, debug=False)
        with torch.no_grad():
            img, _ = GaussianRasterizer(rs)(means3D=sc.t["means3D"], means2D=None,
                                             opacities=sc.t["opacities"], shs=sc.t["shs"],
                                             scales=sc.t["scales"], rotations=sc.t["rotations"])
        host = None
        if self.copy_out:
            host = self.f32.get(img.numel())
            host.copy_(img.reshape(-1), non_blocking=True)
        ev = torch.cuda.Event()
        ev.record()
        return {"ev": ev, "img": img, "host": host, "reqs": reqs}

    def ready(self, h):
        return h["ev"].query()

    def results(self, h):
        r = h["reqs"][0]
        r.result = h["host"].view(3, r.view.height, r.view.width) if self.copy_out else h["img"]
        return [(0, 0)]

    def release(self, h):
        h.clear()

    def recycle(self, req):
        if self.copy_out and req.result is not None:
            self.f32.put(req.result.view(-1))
            req.result = None


def profile_capacity(backend_scenes, resolutions, n_views=4, seed=0, margin=1.3):
    """Seed a CapacityEstimator with exact instance counts of a few random
    views per (scene, resolution) (one geometry pass each)."""
    import torch
    from . import _lib
    from .scenes import random_inside_view
    lib = _lib.load()
    est = CapacityEstimator(margin=margin)
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda")
    stream = _lib.stream_of(dev)
    for si, sc in enumerate(backend_scenes):
        for (w, h) in resolutions:
            for _ in range(n_views):
                v = random_inside_view(rng, w, h)
                keep = [torch.as_tensor(np.asarray(a, np.float32)).to(dev)
                        for a in (np.zeros(3), v.viewmatrix, v.projmatrix, v.campos)]
                view = _lib.DmgsView(w, h, v.tanfovx, v.tanfovy, 1.0, sc.sh_degree, 0, 0,
                                     *[k.data_ptr() for k in keep])
                geom = torch.empty(lib.dmgs_geom_state_bytes(sc.P, w, h), dtype=torch.uint8,
                                   device=dev)
                radii = torch.empty(max(sc.P, 1), dtype=torch.int32, device=dev)
                K = C.c_int64(0)
                _lib.check(lib.dmgs_raster_fwd_geometry(C.byref(view), C.byref(sc.gauss),
                                                        geom.data_ptr(), geom.numel(),
                                                        radii.data_ptr(), C.byref(K), stream),
                           "profile")
                est.observe(Request(-1, si, v, 0.0), K.value)
    return est
