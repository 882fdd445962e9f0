"""Benchmark: forward+backward views/s of the Gaussian rasteriser on the
large-scene workload (3M Gaussians, SH degree 3, scale/rotation inputs).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl dmgs|reference]

A step is one batch of 16 views at 1237x822 rendered forward and backward by
the multi-view batched form (one CUDA-graph replay).  The JSON line (rank 0)
also carries the plain drop-in path on the same scene (one view per call,
the reference's call pattern) and the mixed-resolution batch (16 views of
400x400 / 800x800 / 1237x822 / 1600x900 round-robin) against the plain path
on the same views.  `value` is device-resident throughput; `e2e` is the same
step through the public Python API with the Gaussians and the image
gradients copied from pinned host memory and the images and parameter
gradients copied back inside the timed region.  The reference arm
(--impl reference) times the CPU oracle (FP64 torch restatement of the
reference algorithm) on a bounded sample of the same workload on the host
cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+bwd views/s at 3M Gaussians 1237x822"
MIXED = [(400, 400), (800, 800), (1237, 822), (1600, 900)]
UNIT = "views/s"
WORKLOAD = ("large-scene fwd+bwd: 3M Gaussians, SH3, scale/rotation inputs; step = 16 views at "
            "1237x822, multi-view batched form in a CUDA graph")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="dmgs", choices=["dmgs", "reference"])
    ap.add_argument("--P", type=int, default=3_000_000)
    ap.add_argument("--width", type=int, default=1237)
    ap.add_argument("--height", type=int, default=822)
    ap.add_argument("--views", type=int, default=16, help="views per batch (<= 16)")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-resolution batch")
    ap.add_argument("--no-graph", action="store_true", help="replay without CUDA-graph capture")
    ap.add_argument("--cpu-tiles", type=int, default=24, help="tiles blended in the CPU sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-view-per-call leg")
    ap.add_argument("--no-tune", action="store_true", help="use the default blend configuration")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-loop leg")
    ap.add_argument("--no-mesh", action="store_true", help="skip the mesh-bound training leg")
    ap.add_argument("--no-fc", action="store_true", help="skip the FlexiCubes extraction leg")
    ap.add_argument("--no-tex", action="store_true", help="skip the hash-grid texture leg")
    ap.add_argument("--no-stage2", action="store_true", help="skip the whole stage-2 iteration leg")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="Poisson trace length")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="requests per second")
    ap.add_argument("--serve-budget-gb", type=float, default=16.0, help="HBM budget of in-flight requests")
    ap.add_argument("--serve-burst", type=int, default=800, help="requests of the saturation run")
    return ap.parse_args()


# ----------------------------------------------------------------------------
# clocks
# ----------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------
# CPU oracle sample (reference arm and cpu_baseline)
# ----------------------------------------------------------------------------
def cpu_oracle_sample(scene, view, n_tiles):
    """Time the CPU oracle on a bounded sample of one view: the FP32
    geometry stage over all P Gaussians, then FP64 projection + blending
    forward and backward for `n_tiles` tiles spread over the image.  Returns
    (estimated seconds per full view, description)."""
    import torch
    from oracle import raster as R
    torch.set_num_threads(os.cpu_count() or 1)
    cam = R.Camera(view.width, view.height, view.tanfovx, view.tanfovy, view.viewmatrix,
                   view.projmatrix, view.campos, np.zeros(3, np.float32))
    t0 = time.perf_counter()
    geom = R.geometry_f32(scene.means3D, cam, scene.opacities, scene.scales, scene.rotations)
    t_geom = time.perf_counter() - t0
    gx, gy = cam.grid
    T = gx * gy
    tiles = np.linspace(0, T - 1, n_tiles).astype(np.int64)
    vis = np.nonzero(geom["visible"])[0]
    rect = geom["rect"][vis]
    dbits = geom["depth"][vis].view(np.uint32)
    t1 = time.perf_counter()
    lists = []
    for t in tiles:
        ty, tx = divmod(int(t), gx)
        m = (rect[:, 0] <= tx) & (tx < rect[:, 2]) & (rect[:, 1] <= ty) & (ty < rect[:, 3])
        ids = vis[m]
        order = np.lexsort((ids, dbits[m]))
        lists.append(ids[order])
    t_bin = (time.perf_counter() - t1) * T / n_tiles
    union = np.unique(np.concatenate(lists)) if lists else np.zeros(0, np.int64)
    t2 = time.perf_counter()
    f64 = lambda a: torch.tensor(np.asarray(a, np.float64), requires_grad=True)  # noqa: E731
    leaves = [f64(scene.means3D[union]), f64(scene.opacities[union]), f64(scene.shs[union]),
              f64(scene.scales[union]), f64(scene.rotations[union])]
    sel = torch.arange(len(union))
    ndc, pix, conic, op, rgb = R.project_fp64(cam, leaves[0], leaves[1], shs=leaves[2],
                                              scales=leaves[3], rotations=leaves[4], sel=sel)
    t_proj = time.perf_counter() - t2
    pos = {int(g): i for i, g in enumerate(union)}
    bg = torch.zeros(3, dtype=torch.float64)
    t3 = time.perf_counter()
    total = 0.0
    for t, ids in zip(tiles, lists):
        ty, tx = divmod(int(t), gx)
        x0, y0 = tx * 16, ty * 16
        x1, y1 = min(x0 + 16, cam.width), min(y0 + 16, cam.height)
        yy, xx = torch.meshgrid(torch.arange(y0, y1, dtype=torch.float64),
                                torch.arange(x0, x1, dtype=torch.float64), indexing="ij")
        pxy = torch.stack([xx.reshape(-1), yy.reshape(-1)], 1)
        if len(ids) == 0:
            continue
        g = torch.as_tensor([pos[int(i)] for i in ids])
        out, _, _, _ = R._blend_tile(pxy, pix[g], conic[g], op[g], rgb[g], bg)
        total = total + out.sum()
    if isinstance(total, torch.Tensor):
        total.backward()
    t_blend = (time.perf_counter() - t3) * T / n_tiles
    # projection fwd+bwd scaled to all visible Gaussians
    t_proj_full = t_proj * 3.0 * max(len(vis), 1) / max(len(union), 1)
    est = t_geom + t_bin + t_proj_full + t_blend
    wall = time.perf_counter() - t0
    desc = (f"ESTIMATE, not a whole-view run: FP32 geometry over all {scene.P} Gaussians "
            f"({t_geom:.1f}s) + binning, FP64 projection and blend fwd+bwd on {n_tiles}/{T} tiles "
            f"({len(union)} Gaussians), scaled x{T / n_tiles:.0f} to the full view: {est:.1f}s/view")
    return est, desc, wall, T / n_tiles


def cpu_oracle_cfg1(reps=2):
    """The CPU oracle measured on a whole scene, no extrapolation: the
    plain-rasteriser workload (10,000 Gaussians, SH3, 256x256, FoV 50 deg,
    fwd+bwd with dL/dimage ~ N(0,1)) rendered completely, `reps` times.
    Returns a cpu_baseline-style dict."""
    import torch
    from dmgs_gb300.scenes import small_scene
    from oracle import raster as R
    torch.set_num_threads(os.cpu_count() or 1)
    sc = small_scene()
    v = sc.views[0]
    cam = R.Camera(v.width, v.height, v.tanfovx, v.tanfovy, v.viewmatrix, v.projmatrix, v.campos,
                   np.zeros(3, np.float32))
    dimg = np.random.default_rng(0).standard_normal((3, v.height, v.width)).astype(np.float32)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        ref = R.render(cam, sc.means3D, sc.opacities, shs=sc.shs, scales=sc.scales,
                       rotations=sc.rotations)
        ref.backward(dimg)
        times.append(time.perf_counter() - t0)
    sec = statistics.median(times)
    return {"value": 1.0 / sec, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"MEASURED whole view: {sc.P} Gaussians, SH3, {v.width}x{v.height}, "
                      f"forward + backward of every tile (FP32 geometry, FP64 projection, blend "
                      f"and autograd), median of {reps}: {sec:.2f}s/view"}


# ----------------------------------------------------------------------------
SERVE_SIZES = [200_000, 500_000, 1_000_000, 1_000_000, 2_000_000, 2_000_000, 3_000_000, 3_000_000]
SERVE_RES = [(256, 256), (800, 800), (1237, 822), (1920, 1080)]


def serving_leg(args, dev):
    """Serving loop: 8 resident scenes (the large-scene generator, on the
    device), Poisson arrivals at --serve-rate for --serve-seconds, scene and
    resolution uniform; continuous batching (waves over 4 streams, HBM-budget
    admission) against one-at-a-time plain rendering of the same trace.  A
    saturation run (--serve-burst requests at t=0) gives each mode's
    throughput capacity.  Latency = arrival to the image in host memory."""
    import copy

    from dmgs_gb300.scenes import large_scene_tensors
    from dmgs_gb300.serving import (GpuBackend, PlainBackend, Request, ResidentScene, Scheduler,
                                    poisson_trace, profile_capacity)
    scenes = [ResidentScene(large_scene_tensors(P, 100 + i, dev)) for i, P in enumerate(SERVE_SIZES)]
    est = profile_capacity(scenes, SERVE_RES, n_views=4, seed=5)
    budget = int(args.serve_budget_gb * (1 << 30))
    trace = poisson_trace(args.serve_rate, args.serve_seconds, len(scenes), SERVE_RES, seed=7)
    burst = [Request(i, r.scene, r.view, 0.0)
             for i, r in enumerate(poisson_trace(1000.0, args.serve_burst / 1000.0, len(scenes),
                                                 SERVE_RES, seed=9))]
    fresh = lambda rs: [Request(r.rid, r.scene, r.view, r.arrival) for r in rs]  # noqa: E731
    out = {"scenes_gaussians": SERVE_SIZES, "resolutions": SERVE_RES, "rate_per_s": args.serve_rate,
           "seconds": args.serve_seconds, "requests": len(trace), "budget_gb": args.serve_budget_gb,
           "latency": "arrival to image in pinned host memory"}
    gb = GpuBackend(scenes, arena_bytes=budget, n_streams=4)
    warm = poisson_trace(args.serve_rate, 1.0, len(scenes), SERVE_RES, seed=8)
    Scheduler(gb, budget, estimator=copy.deepcopy(est)).run(warm, deliver=gb.recycle)
    st = Scheduler(gb, budget, estimator=copy.deepcopy(est)).run(fresh(trace), deliver=gb.recycle)
    out["batched"] = st.summary()
    st = Scheduler(gb, budget, estimator=copy.deepcopy(est)).run(fresh(burst), deliver=gb.recycle)
    out["batched_saturated"] = st.summary()
    pb = PlainBackend(scenes)
    one = dict(max_wave=1, max_inflight=1, n_streams=1)
    Scheduler(pb, budget, **one).run(fresh(warm), deliver=pb.recycle)
    st = Scheduler(pb, budget, **one).run(fresh(trace), deliver=pb.recycle)
    out["plain"] = st.summary()
    st = Scheduler(pb, budget, **one).run(fresh(burst), deliver=pb.recycle)
    out["plain_saturated"] = st.summary()
    for k in ("plain", "plain_saturated"):
        out[k].pop("peak_bytes", None)
    out["saturated_ratio_batched_over_plain"] = (out["batched_saturated"]["views_per_s"] /
                                                 out["plain_saturated"]["views_per_s"])
    del scenes, gb, pb
    return out


def mesh_leg(args, dev):
    """Configuration 2: one stage-2 training step (binding -> SH colour ->
    rasteriser with precomputed covariance and colours -> L1 + 0.2 (1 - SSIM)
    -> backward) on the 45,304-face sphere-union-torus mesh, 6 Gaussians per
    face, 800x800, 100 hemisphere cameras, targets rendered from a perturbed
    copy.  Reports steps/s and the binding kernels' achieved GB/s."""
    import torch
    from dmgs_gb300 import _lib
    from dmgs_gb300.meshbound import MeshBoundScene, _gauss_window, sphere_torus_mesh, training_step
    from dmgs_gb300.scenes import hemisphere_views
    lib = _lib.load()
    v, f = sphere_torus_mesh(64)
    scene = MeshBoundScene(v, f, G=6, seed=0, device=dev)
    target = MeshBoundScene(v, f, G=6, seed=0, device=dev)
    gen = torch.Generator(device=dev).manual_seed(11)
    with torch.no_grad():
        target.verts.add_(0.005 * torch.randn(target.verts.shape, device=dev, generator=gen))
        target.features.add_(0.05 * torch.randn(target.features.shape, device=dev, generator=gen))
    views = hemisphere_views(100, 800, 800, seed=0)
    bg = torch.zeros(3, device=dev)
    targets = [target.render(w, bg)[0].detach() for w in views]
    window = _gauss_window(device=dev)
    steps = max(args.steps, 20)
    for i in range(5):
        training_step(scene, views[i], targets[i], bg, window=window)
    torch.cuda.synchronize(dev)
    lib.dmgs_timing_enable(1)
    _lib.timing_collect()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(steps):
        training_step(scene, views[i % len(views)], targets[i % len(views)], bg, window=window)
    e1.record()
    torch.cuda.synchronize(dev)
    lib.dmgs_timing_enable(0)
    kt = _lib.timing_collect()
    ms = e0.elapsed_time(e1) / steps
    # the same step with the loss composed from torch ops (the reference's form)
    for i in range(3):
        training_step(scene, views[i], targets[i], bg, window=window, fused_loss=False)
    e0.record()
    for i in range(steps):
        training_step(scene, views[i % len(views)], targets[i % len(views)], bg, window=window,
                      fused_loss=False)
    e1.record()
    torch.cuda.synchronize(dev)
    ms_torch_loss = e0.elapsed_time(e1) / steps
    # colour and loss both composed from torch ops (the reference's form)
    for i in range(3):
        training_step(scene, views[i], targets[i], bg, window=window, fused_loss=False,
                      fused_color=False)
    e0.record()
    for i in range(steps):
        training_step(scene, views[i % len(views)], targets[i % len(views)], bg, window=window,
                      fused_loss=False, fused_color=False)
    e1.record()
    torch.cuda.synchronize(dev)
    ms_torch_both = e0.elapsed_time(e1) / steps
    F, P, Vn = int(f.shape[0]), scene.P, int(v.shape[0])
    # binding bytes: fwd reads faces (24 B) + 3 vertices (36 B) + per-Gaussian barycentrics
    # (12 B) and writes xyz + covariance (36 B); bwd reads the same geometry and the 36 B
    # of gradients per Gaussian and writes 12 B per vertex
    fwd_bytes = F * (24 + 36) + P * (12 + 36)
    bwd_bytes = F * (24 + 36) + P * (12 + 36) + Vn * 12
    out = {"steps_per_s": 1e3 / ms, "ms_per_step": ms, "faces": F, "gaussians": P,
           "resolution": [800, 800], "cameras": len(views), "steps": steps,
           "loss": "0.8 L1 + 0.2 (1 - SSIM) by the fused loss kernels; sigmoid(SH) colour by "
                   "the fused colour kernel",
           "steps_per_s_torch_loss": 1e3 / ms_torch_loss,
           "steps_per_s_torch_loss_and_colour": 1e3 / ms_torch_both}
    for name, nbytes in (("bind_fwd", fwd_bytes), ("bind_bwd", bwd_bytes)):
        if name in kt:
            t = kt[name][0] / kt[name][1]
            out[name] = {"ms": t, "alg_bytes": nbytes, "achieved_gbs": nbytes / (t * 1e-3) / 1e9}
    if int(os.environ.get("RANK", "0")) == 0 and not getattr(args, "no_cpu", False):
        # the binding's CPU baseline: the oracle's torch restatement of the
        # reference's renew_gaussian / get_covariance_dyn on the same mesh
        import time as _time
        from oracle import binding as obind  # CPU baseline only
        torch.set_num_threads(os.cpu_count())
        vc = v.detach().cpu().double().requires_grad_(True)
        sfc = torch.full((1,), 0.5493, dtype=torch.float64, requires_grad=True)
        bcc = scene.bc.detach().cpu().double()
        rad = scene.rad_base
        reps = 3
        t0 = _time.perf_counter()
        for _ in range(reps):
            xyz_c, cov_c, _, _ = obind.bind_stage2(vc, f.cpu(), bcc, rad, 1e-6, sfc)
            (xyz_c.sum() + cov_c.sum()).backward()
        out["binding_cpu_baseline"] = {
            "fwd_bwd_ms": (_time.perf_counter() - t0) / reps * 1e3, "cores": os.cpu_count(),
            "kind": "port", "sample": "float64 torch restatement of the stage-2 binding on the host, "
                                      f"{F} faces x 6 Gaussians, 3 forward+backward"}
    for name in ("preprocess", "blend_fwd", "blend_bwd", "preprocess_bwd", "sh_colors", "l1_ssim"):
        if name in kt:
            out.setdefault("kernels_ms", {})[name] = kt[name][0] / kt[name][1]
    del scene, target, targets
    return out


def flexicubes_leg(args, dev):
    """FlexiCubes extraction as stage 2 runs it every step
    (scene/gaussian_geo_model_mlp_flex.py:240-255: deformed grid, per-cube
    weights initialised to ones, training mode) on the sphere-union-torus
    field over [-1,1]^3: forward and forward+backward ms at 64^3 (the
    configuration-2 grid) and at 128^3 and 250^3 (the reference configs'
    res_fg range, 100-300), with the float32 CPU oracle at 64^3 beside it."""
    import torch
    from dmgs_gb300 import _lib
    from dmgs_gb300.flexicubes import FlexiCubes
    from dmgs_gb300.meshbound import sdf_sphere_torus
    lib = _lib.load()
    fc = FlexiCubes(device=dev)
    out = {"field": "sphere(0.6) union torus(0.7, 0.2) over [-1,1]^3, training mode, "
                    "deformation tanh(0), raw weights 1 (the reference's initialisation)"}
    for res in (64, 128, 250):
        grid, cubes = fc.construct_voxel_grid_v2(res, [-1.0] * 3, [1.0] * 3)
        s0 = torch.as_tensor(sdf_sphere_torus(grid.double().cpu().numpy()), dtype=torch.float32,
                             device=dev)
        sdf = s0.clone().requires_grad_(True)
        deform = torch.zeros_like(grid, requires_grad=True)
        w = torch.ones((cubes.shape[0], 21), device=dev, requires_grad=True)
        maxd = 2.0 / res / 4

        def fwd():
            x = grid + maxd * torch.tanh(deform)
            return fc(x, sdf, cubes, res, w[:, :12], w[:, 12:20], w[:, 20], training=True)

        def step(i):
            v, f, L, se = fwd()
            (v.square().sum() + L.mean()).backward()

        n = 20
        ms_fwd = timed(lambda i: fwd(), n, 3, dev) / n
        l0 = lib.dmgs_kernel_launches()
        ms_step = timed(step, n, 3, dev) / n
        launches = (lib.dmgs_kernel_launches() - l0) / (n + 3)
        lib.dmgs_timing_enable(1)
        _lib.timing_collect()
        for i in range(5):
            step(i)
        torch.cuda.synchronize(dev)
        lib.dmgs_timing_enable(0)
        kt = _lib.timing_collect()
        v, f, L, se = fwd()
        out[f"res{res}"] = {"cubes": int(cubes.shape[0]), "faces": int(f.shape[0]),
                            "vertices": int(v.shape[0]), "surface_edges": int(se.shape[0]),
                            "fwd_ms": ms_fwd, "fwd_bwd_ms": ms_step,
                            "own_kernels_per_fwd_bwd": launches,
                            "kernel_ms_per_step": {k: kt[k][0] / 5 for k in ("fc_fwd", "fc_bwd")
                                                   if k in kt}}
        del grid, cubes, s0, sdf, deform, w, v, f, L, se
    if int(os.environ.get("RANK", "0")) == 0 and not args.no_cpu:
        from oracle import flexicubes as ofc  # CPU baseline only
        torch.set_num_threads(os.cpu_count())
        verts, cubes = ofc.voxel_grid(64, (-1, -1, -1), (1, 1, 1))
        s = torch.tensor(sdf_sphere_torus(verts.double().numpy()), dtype=torch.float32,
                         requires_grad=True)
        wc = torch.ones((cubes.shape[0], 21), requires_grad=True)
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            v, f, L, se = ofc.extract(verts, s, cubes, 64, wc[:, :12], wc[:, 12:20], wc[:, 20],
                                      training=True)
            (v.square().sum() + L.mean()).backward()
        out["cpu_baseline"] = {"fwd_bwd_ms": (time.perf_counter() - t0) / reps * 1e3,
                               "res": 64, "cores": os.cpu_count(), "kind": "port",
                               "sample": "float32 torch oracle on the host, 3 forward+backward"}
    return out


def stage2_leg(args, dev):
    """The reference's whole stage-2 iteration (train_geo_stage2.py:101-135)
    on the library's kernels: FlexiCubes at 64^3 every step (learnable SDF,
    deformation, per-cube weights; training mode) -> binding (6 Gaussians per
    face, shared table) -> hash-grid texture SH features -> sigmoid(SH)
    colours -> rasteriser (800x800, 100 hemisphere cameras) -> L1 + SSIM +
    the SDF and FlexiCubes regularisers -> backward into every learnable.
    Steps/s (forward + backward, no optimiser) and the kernels' share."""
    import torch
    from dmgs_gb300 import _lib
    from dmgs_gb300.meshbound import Stage2Model
    from dmgs_gb300.scenes import hemisphere_views
    lib = _lib.load()
    model = Stage2Model(res=64, device=dev)
    views = hemisphere_views(100, 800, 800, seed=0)
    bg = torch.zeros(3, device=dev)
    with torch.no_grad():
        saved = model.texture.encoder.params.clone()
        gen = torch.Generator(device=dev).manual_seed(5)
        model.texture.encoder.params.add_(0.05 * torch.randn(saved.shape, device=dev, generator=gen))
        targets = [model.render(w, bg)[0].detach() for w in views[:20]]
        model.texture.encoder.params.copy_(saved)
        faces = int(model.mesh()[1].shape[0])
    steps = max(args.steps, 20)
    ms = timed(lambda i: model.step(views[i % 20], targets[i % 20], bg), steps, 5, dev) / steps
    lib.dmgs_timing_enable(1)
    _lib.timing_collect()
    for i in range(5):
        model.step(views[i], targets[i], bg)
    torch.cuda.synchronize(dev)
    lib.dmgs_timing_enable(0)
    kt = _lib.timing_collect()
    return {"steps_per_s": 1e3 / ms, "ms_per_step": ms, "grid": 64, "faces": faces,
            "gaussians": faces * 6, "resolution": [800, 800], "steps": steps,
            "kernel_ms_per_step": {k: v[0] / 5 for k, v in sorted(kt.items())}}


def texture_leg(args, dev):
    """The stage-2 hash-grid texture query (MLPTexture3D.sample_noact,
    scene/gaussian_geo_model_mlp_flex.py:313) at the configuration-2
    Gaussian count: 271,824 points on the 45,304-face FlexiCubes mesh
    (6 per face at Dirichlet(1,1,1) barycentrics), 48 SH channels, AABB =
    the mesh bounds x 1.1 (:206-208).  Forward and forward+backward ms."""
    import torch
    from dmgs_gb300 import _lib
    from dmgs_gb300.meshbound import sphere_torus_mesh
    from dmgs_gb300.texture import MLPTexture3D
    lib = _lib.load()
    v, f = sphere_torus_mesh(64)
    gen = torch.Generator(device=dev).manual_seed(3)
    bc = torch.distributions.Dirichlet(torch.ones(3, device=dev)).sample((f.shape[0] * 6,))
    tri = v[f].repeat_interleave(6, 0)
    xyz = (bc.unsqueeze(2) * tri).sum(1).contiguous().requires_grad_(True)
    aabb = torch.stack([v.min(0).values, v.max(0).values]) * 1.1
    tex = MLPTexture3D(aabb, channels=48, device=dev)
    up = torch.randn((xyz.shape[0], 48), device=dev, generator=gen)

    def step(i):
        out = tex.sample_noact(xyz)
        (out * up).sum().backward()

    n = 20
    with torch.no_grad():
        ms_fwd = timed(lambda i: tex.sample_noact(xyz), n, 3, dev) / n
    l0 = lib.dmgs_kernel_launches()
    ms_step = timed(step, n, 3, dev) / n
    launches = (lib.dmgs_kernel_launches() - l0) / (n + 3)
    lib.dmgs_timing_enable(1)
    _lib.timing_collect()
    for i in range(5):
        step(i)
    torch.cuda.synchronize(dev)
    lib.dmgs_timing_enable(0)
    kt = _lib.timing_collect()
    out = {"points": int(xyz.shape[0]), "channels": 48, "fwd_ms": ms_fwd, "fwd_bwd_ms": ms_step,
           "own_kernels_per_fwd_bwd": launches,
           "kernel_ms_per_step": {k: kt[k][0] / 5 for k in ("tex_fwd", "tex_bwd", "tex_scatter")
                                  if k in kt},
           "adjoint_split": "tex_bwd = MLP adjoint incl. the weight-gradient GEMMs; tex_scatter = "
                            "table and position gradients (float2 atomics)",
           "table_mb": tex.encoder.params.numel() * 4 / 1e6,
           "encoding": "float32 hash grid (the reference's tiny-cuda-nn default is half)"}
    if int(os.environ.get("RANK", "0")) == 0 and not args.no_cpu:
        from oracle import texture as otex  # CPU baseline only
        torch.set_num_threads(os.cpu_count())
        m = 32768
        x = xyz[:m].detach().cpu().requires_grad_(True)
        tb = tex.encoder.params.detach().cpu().view(-1, 2).requires_grad_(True)
        W = [w.detach().cpu().requires_grad_(True) for w in tex.net.weights()]
        t0 = time.perf_counter()
        o = otex.sample_noact(x, aabb.cpu(), tb, W)
        (o * up[:m].cpu()).sum().backward()
        out["cpu_baseline"] = {"fwd_bwd_ms_per_271824_points": (time.perf_counter() - t0) * 1e3 *
                               xyz.shape[0] / m, "cores": os.cpu_count(), "kind": "port",
                               "sample": f"float32 torch oracle, {m} points, scaled to 271,824"}
    return out


def bytes_model(name, P, V, K, npix, nviews=1, K1=None):
    """Algorithmic DRAM bytes per launch (SH3, scale/rotation inputs).  For
    a batched launch V, K, npix (and K1, the row-list entries) are sums over
    the views."""
    if name == "batch_preprocess":
        return P * (12 + 16 + 12 + 4 + 192) + nviews * P * 4 + V * 48
    if name == "batch_preprocess_bwd":
        return P * (236 + 236) + V * 48
    if name == "preprocess":
        return P * 12 + V * (12 + 16 + 4 + 192) + P * 4 + V * 48
    if name == "blend_fwd":
        return K * 40 + npix * 20
    if name == "blend_bwd":
        return K * 40 + npix * 20 + P * 36
    if name == "preprocess_bwd":
        return P * (236 + 36 + 236)
    if name == "bin_depth_sort":  # 4 LSD passes over (depth bits, index): 4 B read by the
        return V * 80             # histogram, 8 B read + 8 B written by the scatter, per key
    if name == "bin_compact":
        return P * nviews + V * 12
    if name == "bin_emit":  # row lists read (8 B per entry), tile lists written (4 B per instance)
        return None if K1 is None else K * 4 + K1 * 8
    if name == "bin_row_emit":  # sorted rectangles + indices read, row lists written
        return None if K1 is None else V * 12 + K1 * 8
    return None



def job_time_ms(ms_local, world, device):
    """The job's timed-region length: the max over ranks of each rank's own
    (every rank runs the same steps; the job ends with the slowest).  One
    all-reduce over the default process group when world > 1."""
    if world <= 1:
        return ms_local
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms_job, world, views_per_step, steps):
    """Whole-job views/s of `world` independent replicas (weak scaling)."""
    return world * views_per_step * steps / (ms_job / 1e3)


def timed(fn, steps, warmup, sync_dev):
    """Run fn(i) warmup times, then time `steps` calls with CUDA events."""
    import torch
    for i in range(warmup):
        fn(i)
    torch.cuda.synchronize(sync_dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(steps):
        fn(i)
    e1.record()
    torch.cuda.synchronize(sync_dev)
    return e0.elapsed_time(e1)


def kernel_table(kt, model_args):
    kernels = {}
    tot_all = sum(x[0] for x in kt.values()) or 1e-9
    for name, (tot, n) in kt.items():
        avg = tot / max(n, 1)
        b = bytes_model(name, *model_args)
        kernels[name] = {"launches": n, "total_ms": round(tot, 4), "avg_ms": round(avg, 5),
                         "share": round(tot / tot_all, 4)}
        if b is not None:
            kernels[name]["alg_bytes"] = int(b)
            kernels[name]["achieved_gbs"] = round(b / (avg / 1e3) / 1e9, 1)
        if name == "bin_depth_sort":
            kernels[name]["keys_per_s"] = round(model_args[1] / (avg / 1e3), 1)
    return kernels


def blend_config(cfg):
    from dmgs_gb300.batched import TILE_SHAPES
    return {"pixels_per_thread": cfg[0], "gaussians_per_batch": cfg[1],
            "cta_shape": TILE_SHAPES[cfg[2] if len(cfg) > 2 else 0]}


def summary_of(line):
    """The headline figure of every leg in a few hundred bytes, printed as the
    line's last key so that a reader of only the line's end still sees them."""
    r = lambda x, n=1: None if x is None else round(x, n)  # noqa: E731
    s = {"views_per_s": r(line["value"]), "ms_per_step": r(line["ms_per_step"], 3)}
    pl, mx, sv = line.get("plain"), line.get("mixed"), line.get("serving")
    if pl:
        s["plain_views_per_s"] = r(pl["views_per_s"])
        s["batched_over_plain"] = r(pl.get("ratio_batched_over_plain"), 3)
    if mx:
        s["mixed_views_per_s"] = r(mx["batched_views_per_s"])
        s["mixed_plain_views_per_s"] = r(mx.get("plain_views_per_s"))
    if line.get("e2e"):
        s["e2e_views_per_s"] = r(line["e2e"]["value"])
    if line.get("roofline"):
        s["roofline"] = f'{line["roofline"]["kernel"]} {line["roofline"]["frac"]}'
    if line.get("kernels"):
        s["kernel_ms"] = {k: r(v["avg_ms"], 3) for k, v in line["kernels"].items()}
    if sv:
        s["serving_p50_p99_ms"] = [r(sv["batched"]["p50_ms"], 3), r(sv["batched"]["p99_ms"], 3)]
        s["serving_plain_p50_p99_ms"] = [r(sv["plain"]["p50_ms"], 3), r(sv["plain"]["p99_ms"], 3)]
        s["serving_saturated_views_per_s"] = [r(sv["batched_saturated"]["views_per_s"]),
                                              r(sv["plain_saturated"]["views_per_s"])]
    if line.get("mesh_training"):
        s["mesh_steps_per_s"] = r(line["mesh_training"]["steps_per_s"])
    if line.get("stage2_full"):
        s["stage2_steps_per_s"] = r(line["stage2_full"]["steps_per_s"])
    if line.get("texture"):
        s["texture_fwd_bwd_ms"] = r(line["texture"]["fwd_bwd_ms"], 3)
    if line.get("flexicubes"):
        s["flexicubes_fwd_bwd_ms"] = {k: r(v["fwd_bwd_ms"], 3) for k, v in line["flexicubes"].items()
                                      if k.startswith("res")}
    return s


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    from dmgs_gb300.scenes import large_scene
    if args.impl == "reference":
        if rank != 0:
            return
        scene = large_scene(P=args.P, seed=0, n_views=4, width=args.width, height=args.height)
        times, walls = [], []
        desc, factor = "", 1.0
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            est, desc, _, factor = cpu_oracle_sample(scene, scene.views[i % len(scene.views)],
                                                     args.cpu_tiles)
            if i >= args.warmup:
                times.append(est)
                walls.append(time.perf_counter() - t0)
        v = 1.0 / statistics.mean(times)
        cfg1 = cpu_oracle_cfg1()
        print(json.dumps({
            "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(walls),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": (f"CPU oracle (FP64 torch restatement of the rasteriser) on the "
                                    f"host cores; a step is ONE sampled view of the large scene "
                                    f"({args.P} Gaussians, SH3, {args.width}x{args.height}): FP32 "
                                    f"geometry of every Gaussian, FP64 projection and blend "
                                    f"fwd+bwd on {args.cpu_tiles} tiles; `value` scales that "
                                    f"sample x{factor:.0f} to a whole view (an estimate)"),
                       "P": args.P, "width": args.width, "height": args.height,
                       "views_per_step": 1, "tiles_sampled": args.cpu_tiles,
                       "extrapolation_factor": round(factor, 2), "parallelism": "host cores",
                       "graph": False},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": desc, "measured_cfg1": cfg1},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    import torch
    import dmgs_gb300
    from dmgs_gb300 import _lib
    from dmgs_gb300.batched import BatchedRasterizer, autotune
    from dmgs_gb300.scenes import random_inside_view

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    lib = _lib.load()
    nv = max(1, min(16, args.views))

    scene = large_scene(P=args.P, seed=rank, n_views=nv, width=args.width, height=args.height)
    P = scene.P
    t = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    g = {"means3D": t(scene.means3D), "opacities": t(scene.opacities), "shs": t(scene.shs),
         "scales": t(scene.scales), "rotations": t(scene.rotations)}

    def settings_of(v):
        return dmgs_gb300.GaussianRasterizationSettings(
            image_height=v.height, image_width=v.width, tanfovx=v.tanfovx, tanfovy=v.tanfovy,
            bg=torch.zeros(3, device=dev), scale_modifier=1.0, viewmatrix=t(v.viewmatrix),
            projmatrix=t(v.projmatrix), sh_degree=3, campos=t(v.campos), prefiltered=False,
            debug=False)

    settings = [settings_of(v) for v in scene.views]
    gen = torch.Generator(device=dev).manual_seed(0)
    dimgs = [torch.randn(3, s.image_height, s.image_width, device=dev, generator=gen) for s in settings]
    leaves = {k: v.clone().requires_grad_(True) for k, v in g.items()}

    def plain_step(i, sets, douts, tensors=leaves):
        m2 = torch.zeros_like(tensors["means3D"], requires_grad=True)
        img, radii = dmgs_gb300.GaussianRasterizer(sets[i % len(sets)])(
            means3D=tensors["means3D"], means2D=m2, opacities=tensors["opacities"],
            shs=tensors["shs"], scales=tensors["scales"], rotations=tensors["rotations"])
        img.backward(douts[i % len(douts)])
        for p in tensors.values():
            p.grad = None
        return img, m2

    clocks = ClockSampler(local)
    clocks.start()
    # ---------------- plain drop-in path: one view per call ----------------
    plain = None
    if not args.no_plain:
        lib.dmgs_timing_enable(0)
        _lib.timing_collect()
        lib.dmgs_timing_enable(1)
        n0 = lib.dmgs_kernel_launches()
        ms_plain = timed(lambda i: plain_step(i, settings, dimgs), args.steps, args.warmup, dev)
        lib.dmgs_timing_enable(0)
        kt_plain = _lib.timing_collect()
        plain = {"views_per_s": args.steps / (ms_plain / 1e3), "ms_per_view": ms_plain / args.steps,
                 "launches_per_view": (lib.dmgs_kernel_launches() - n0) / (args.steps + args.warmup)}

    # ---------------- batched form: 16 views per step, CUDA graph ----------------
    br = BatchedRasterizer(settings, g, means2D_grads=False, densify_stats=True)
    for d, s in zip(br.dL_dout, dimgs):
        d.copy_(s)
    tune = None
    if not args.no_tune:
        tune = autotune(br, iters=3, cache_path=os.environ.get("DMGS_AUTOTUNE_CACHE"))
    counts = br.count_instances()
    br.forward()
    bin_counters = br.counters()
    K1_sum = sum(c["K1"] for c in bin_counters)
    lib.dmgs_timing_enable(1)
    _lib.timing_collect()
    n0 = lib.dmgs_kernel_launches()
    br.step()  # eager, instrumented: per-kernel times of one batch
    torch.cuda.synchronize(dev)
    launches_per_step = lib.dmgs_kernel_launches() - n0
    lib.dmgs_timing_enable(0)
    kt_batch = _lib.timing_collect()
    if not args.no_graph:
        br.capture()
    if world > 1:
        torch.distributed.barrier()
    ms_batch = timed(lambda i: br.step(), args.steps, args.warmup, dev)
    br.status()  # raises on a capacity overflow
    ms_batch = job_time_ms(ms_batch, world, dev)
    value = replica_value(ms_batch, world, nv, args.steps)

    # ---------------- mixed resolutions (16 views) ----------------
    mixed = None
    if not args.no_mixed:
        rng = np.random.default_rng(1234 + rank)
        mviews = [random_inside_view(rng, *MIXED[i % len(MIXED)]) for i in range(nv)]
        msets = [settings_of(v) for v in mviews]
        mdouts = [torch.randn(3, s.image_height, s.image_width, device=dev, generator=gen) for s in msets]
        ms_mplain = None if args.no_plain else timed(lambda i: plain_step(i, msets, mdouts), nv, 2, dev)
        bm = BatchedRasterizer(msets, g, means2D_grads=False, densify_stats=True)
        for d, s in zip(bm.dL_dout, mdouts):
            d.copy_(s)
        mtune = None
        if not args.no_tune:
            mtune = autotune(bm, iters=3, cache_path=os.environ.get("DMGS_AUTOTUNE_CACHE"))
        if not args.no_graph:
            bm.capture()
        ms_mb = timed(lambda i: bm.step(), args.steps, args.warmup, dev)
        bm.status()
        mixed = {"views": nv, "resolutions": MIXED,
                 "batched_views_per_s": nv * args.steps / (ms_mb / 1e3),
                 "blend_config": blend_config(bm.cfg),
                 "autotune": mtune and {"best": mtune["best"], "axes": mtune.get("axes"),
                                        "ms": mtune["ms"]}}
        if ms_mplain is not None:
            mixed["plain_views_per_s"] = nv / (ms_mplain / 1e3)
            mixed["ratio_batched_over_plain"] = (nv * args.steps / ms_mb) / (nv / ms_mplain)
        del bm
    clk = clocks.stop()

    # ---------------- roofline of the dominant kernel (batched step) ----------------
    Vs = sum(int((r > 0).sum()) for r in br.radii)
    npix = sum(s.image_width * s.image_height for s in settings)
    kernels = kernel_table(kt_batch, (P, Vs, sum(counts), npix, nv, K1_sum))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    roof = None
    if kt_batch:
        dom = max(kt_batch.items(), key=lambda kv: kv[1][0])[0]
        traffic = None
        try:
            traffic = json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(dom)
        except Exception:
            pass
        if kernels[dom].get("alg_bytes"):
            ach = kernels[dom]["achieved_gbs"]
            roof = {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                    "frac": round(ach / hbm_peak, 4), "traffic": traffic, "peak_source": peak_src}

    # ---------------- e2e: host buffers through the public API ----------------
    # HostPipeline: every step uploads the Gaussians and image gradients from
    # pinned host memory and downloads the images and parameter gradients;
    # uploads/downloads of neighbouring steps overlap the current step's
    # compute (two ping-pong device buffer sets, copy streams).
    e2e = None
    if not args.no_e2e:
        from dmgs_gb300.batched import HostPipeline
        names = ["means3D", "opacities", "shs", "scales", "rotations"]
        pipe = HostPipeline(settings, g, names, means2D_grads=False, densify_stats=True,
                            cfg=tuple(br.cfg))
        host_in = {k: g[k].cpu().pin_memory() for k in names}
        host_dout = [d.cpu().pin_memory() for d in dimgs]
        host_img = [[torch.empty(i.shape).pin_memory() for i in br.images] for _ in range(2)]
        host_grad = [{k: torch.empty(br.grads[k].shape).pin_memory() for k in names}
                     for _ in range(2)]
        n_e2e = max(3, args.steps)  # the same step count as the main leg (fill and drain included)

        def e2e_run(n):
            pipe.start()
            for i in range(n):
                pipe.submit(host_in, host_dout, host_img[i % 2], host_grad[i % 2])
            pipe.finish()

        e2e_run(2)  # warm-up
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        e2e_run(n_e2e)
        e1.record()
        torch.cuda.synchronize(dev)
        ems = job_time_ms(e0.elapsed_time(e1), world, dev)
        h2d = sum(h.numel() * 4 for h in host_in.values()) + sum(h.numel() * 4 for h in host_dout)
        d2h = (sum(h.numel() * 4 for h in host_img[0]) +
               sum(h.numel() * 4 for h in host_grad[0].values()))
        e2e = {"value": replica_value(ems, world, nv, n_e2e), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": n_e2e, "views_per_step": nv,
               "api": "dmgs_gb300.batched.HostPipeline (uploads and downloads of neighbouring "
                      "steps overlap the current step), pinned host buffers"}
        del pipe

    br_cfg = br.cfg
    serving = None
    if not args.no_serve:
        del br
        torch.cuda.empty_cache()
        clocks_s = ClockSampler(local)
        clocks_s.start()
        serving = serving_leg(args, dev)
        serving["clocks"] = clocks_s.stop()

    mesh = None
    if not args.no_mesh:
        mesh = mesh_leg(args, dev)
    fcl = None
    if not args.no_fc:
        fcl = flexicubes_leg(args, dev)
    texl = None
    if not args.no_tex:
        texl = texture_leg(args, dev)
    st2 = None
    if not args.no_stage2:
        st2 = stage2_leg(args, dev)

    cpu = None
    if rank == 0 and not args.no_cpu:
        est, desc, _, _ = cpu_oracle_sample(scene, scene.views[0], args.cpu_tiles)
        cpu = {"value": 1.0 / est, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": desc, "measured_cfg1": cpu_oracle_cfg1()}

    if rank == 0:
        Kp = statistics.mean(counts)
        in_mb = sum(v.numel() * v.element_size() for v in g.values()) / 1e6
        l2_note = (f"inputs ({in_mb:.0f} MB) larger than L2" if in_mb > 129 else
                   f"inputs ({in_mb:.0f} MB) smaller than L2: not a bench configuration")
        if plain is not None:
            plain["ratio_batched_over_plain"] = value / max(plain["views_per_s"], 1e-9)
            plain["kernels"] = kernel_table(kt_plain, (P, Vs / nv, Kp, npix / nv, 1, K1_sum / nv))
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_batch / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "P": P, "width": args.width, "height": args.height,
                       "views_per_step": nv, "parallelism": "replicas" if world > 1 else "1 gpu",
                       "outputs": "images, parameter gradients summed over views, densification "
                                  "statistics (fused add_densification_stats)",
                       "l2": l2_note, "mean_instances_K": int(Kp),
                       "mean_row_entries_K1": int(K1_sum / nv),
                       "blend_config": blend_config(br_cfg),
                       "graph": not args.no_graph},
            "plain": plain,
            "mixed": mixed,
            "autotune": tune and {"best": tune["best"], "axes": tune.get("axes"), "ms": tune["ms"]},
            "roofline": roof, "kernels": kernels, "cpu_baseline": cpu, "e2e": e2e,
            "serving": serving, "mesh_training": mesh, "flexicubes": fcl,
            "texture": texl, "stage2_full": st2,
            "gpu_launches": int(launches_per_step * args.steps), "clocks": clk}
        line["summary"] = summary_of(line)  # last key: the headline figures of every leg
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
