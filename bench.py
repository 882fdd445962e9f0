"""Benchmark: forward+backward views/s of the Gaussian rasteriser on the
large-scene workload (3M Gaussians, 1237x822, SH degree 3, scale/rotation
inputs), one view per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl dmgs|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput;
`e2e` is the same metric through the drop-in API with the step's inputs
copied from pinned host memory and its image + gradients copied back inside
the timed region.  The reference arm (--impl reference) times the CPU oracle
(FP64 torch restatement of the reference algorithm) on a bounded sample of
the same workload on the host cores.
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
UNIT = "views/s"
WORKLOAD = "large-scene fwd+bwd: 3M Gaussians, 1237x822, SH3, scale/rotation inputs, 1 view/step"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="dmgs", choices=["dmgs", "reference"])
    ap.add_argument("--P", type=int, default=3_000_000)
    ap.add_argument("--width", type=int, default=1237)
    ap.add_argument("--height", type=int, default=822)
    ap.add_argument("--views", type=int, default=8, help="distinct camera poses cycled over steps")
    ap.add_argument("--cpu-tiles", type=int, default=24, help="tiles blended in the CPU sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
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
    desc = (f"FP32 geometry over all {scene.P} Gaussians ({t_geom:.1f}s) + binning, FP64 projection "
            f"and blend fwd+bwd on {n_tiles}/{T} tiles ({len(union)} Gaussians), scaled to the full "
            f"view: {est:.1f}s/view")
    return est, desc


# ----------------------------------------------------------------------------
def bytes_model(name, P, V, K, npix):
    """Algorithmic DRAM bytes per launch (SH3, scale/rotation inputs)."""
    if name == "preprocess":
        return P * 12 + V * (12 + 16 + 4 + 192) + P * 4 + V * 48
    if name == "blend_fwd":
        return K * 40 + npix * 20
    if name == "blend_bwd":
        return K * 40 + npix * 20 + P * 36
    if name == "preprocess_bwd":
        return P * (236 + 36 + 236)
    if name == "segment_sort":
        return K * 12
    if name == "scatter":
        return K * 8 + V * 16
    return None


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    from dmgs_gb300.scenes import large_scene
    if args.impl == "reference":
        if rank != 0:
            return
        scene = large_scene(P=args.P, seed=0, n_views=max(args.views, 1), width=args.width,
                            height=args.height)
        times = []
        desc = ""
        for i in range(args.warmup + args.steps):
            est, desc = cpu_oracle_sample(scene, scene.views[i % len(scene.views)], args.cpu_tiles)
            if i >= args.warmup:
                times.append(est)
        v = 1.0 / statistics.mean(times)
        print(json.dumps({
            "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "P": args.P, "width": args.width, "height": args.height},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": desc},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    import torch
    import dmgs_gb300
    from dmgs_gb300 import _lib

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    _lib.load()

    scene = large_scene(P=args.P, seed=rank, n_views=args.views, width=args.width, height=args.height)
    P = scene.P
    t = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    xyz = t(scene.means3D).requires_grad_(True)
    opac = t(scene.opacities).requires_grad_(True)
    shs = t(scene.shs).requires_grad_(True)
    scales = t(scene.scales).requires_grad_(True)
    rots = t(scene.rotations).requires_grad_(True)
    settings = []
    for v in scene.views:
        settings.append(dmgs_gb300.GaussianRasterizationSettings(
            image_height=v.height, image_width=v.width, tanfovx=v.tanfovx, tanfovy=v.tanfovy,
            bg=torch.zeros(3, device=dev), scale_modifier=1.0, viewmatrix=t(v.viewmatrix),
            projmatrix=t(v.projmatrix), sh_degree=3, campos=t(v.campos), prefiltered=False,
            debug=False))
    gen = torch.Generator(device=dev)
    gen.manual_seed(0)
    dimg = torch.randn(3, args.height, args.width, device=dev, generator=gen)

    def step(i, tensors=None):
        x, o, s, sc, r = tensors if tensors is not None else (xyz, opac, shs, scales, rots)
        m2 = torch.zeros_like(x, requires_grad=True)
        img, radii = dmgs_gb300.GaussianRasterizer(settings[i % len(settings)])(
            means3D=x, means2D=m2, opacities=o, shs=s, scales=sc, rotations=r)
        img.backward(dimg)
        return img, radii, m2

    def zero_grads(ts):
        for p in ts:
            p.grad = None

    for i in range(args.warmup):
        step(i)
        zero_grads([xyz, opac, shs, scales, rots])
    torch.cuda.synchronize()

    # per-view instance counts (for the byte model)
    stats = []
    for i in range(len(settings)):
        with torch.no_grad():
            img, radii = dmgs_gb300.GaussianRasterizer(settings[i])(
                means3D=xyz.detach(), means2D=torch.zeros_like(xyz), opacities=opac.detach(),
                shs=shs.detach(), scales=scales.detach(), rotations=rots.detach())
        stats.append(int((radii > 0).sum()))
    torch.cuda.synchronize()

    # ---------------- timed region: device-resident inputs ----------------
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    _lib.timing_collect()
    _lib.timing_enable(True)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for i in range(args.steps):
        step(i)
        zero_grads([xyz, opac, shs, scales, rots])
    ev1.record()
    torch.cuda.synchronize()
    _lib.timing_enable(False)
    kt = _lib.timing_collect()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        tt = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms = float(tt.item())
    value = world * args.steps / (ms / 1e3)

    # K per view from the forward state is not exposed by the drop-in; the
    # byte model uses the measured instance count of each view.
    Ks = []
    for i in range(len(settings)):
        rs = settings[i]
        from dmgs_gb300._lib import DmgsGaussians, ptr
        from dmgs_gb300.rasterizer import make_view
        import ctypes as C
        keep = []
        view = make_view(rs, dev, keep)
        g = DmgsGaussians(P, 16, ptr(xyz), ptr(opac), ptr(shs), None, ptr(scales), ptr(rots), None)
        lib = _lib.load()
        geom = torch.empty(lib.dmgs_geom_state_bytes(P, args.width, args.height), dtype=torch.uint8, device=dev)
        radii = torch.empty(P, dtype=torch.int32, device=dev)
        K = C.c_int64(0)
        _lib.check(lib.dmgs_raster_fwd_geometry(view, g, geom.data_ptr(), geom.numel(), radii.data_ptr(),
                                                C.byref(K), _lib.stream_of(dev)), "bench K")
        Ks.append(int(K.value))
    steps_views = [i % len(settings) for i in range(args.steps)]
    K_avg = statistics.mean(Ks[i] for i in steps_views)
    V_avg = statistics.mean(stats[i] for i in steps_views)
    npix = args.width * args.height
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    kernels = {}
    for name, (tot, n) in kt.items():
        avg = tot / max(n, 1)
        b = bytes_model(name, P, V_avg, K_avg, npix)
        kernels[name] = {"launches": n, "total_ms": round(tot, 4), "avg_ms": round(avg, 5),
                         "share": round(tot / max(sum(x[0] for x in kt.values()), 1e-9), 4)}
        if b is not None:
            kernels[name]["alg_bytes"] = int(b)
            kernels[name]["achieved_gbs"] = round(b / (avg / 1e3) / 1e9, 1)
    dom = max(kt.items(), key=lambda kv: kv[1][0])[0] if kt else None
    roof = None
    if dom is not None and kernels[dom].get("alg_bytes"):
        ach = kernels[dom]["achieved_gbs"]
        traffic = None
        try:
            prof = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
            traffic = prof.get(dom)
        except Exception:
            pass
        roof = {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                "frac": round(ach / hbm_peak, 4), "traffic": traffic,
                "peak_source": peak_src}
    launches = sum(n for (_, n) in kt.values())

    # ---------------- e2e: host buffers through the drop-in API ----------------
    e2e = None
    if not args.no_e2e:
        host = [torch.tensor(a).pin_memory() for a in
                (scene.means3D, scene.opacities, scene.shs, scene.scales, scene.rotations)]
        out_img = torch.empty(3, args.height, args.width).pin_memory()
        out_g = [torch.empty_like(h).pin_memory() for h in host]
        h2d = sum(h.numel() * 4 for h in host)
        d2h = out_img.numel() * 4 + sum(h.numel() * 4 for h in host) + P * 12
        out_m2 = torch.empty(P, 3).pin_memory()
        n_e2e = max(3, min(args.steps, 10))

        def e2e_step(i):
            dv = [h.to(dev, non_blocking=True).requires_grad_(True) for h in host]
            img, radii, m2 = step(i, dv)
            out_img.copy_(img.detach(), non_blocking=True)
            for o, d in zip(out_g, dv):
                o.copy_(d.grad, non_blocking=True)
            out_m2.copy_(m2.grad, non_blocking=True)

        for i in range(2):
            e2e_step(i)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(n_e2e):
            e2e_step(i)
        e1.record()
        torch.cuda.synchronize()
        ems = e0.elapsed_time(e1)
        e2e = {"value": world * n_e2e / (ems / 1e3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": n_e2e,
               "api": "dmgs_gb300.GaussianRasterizer (drop-in), pinned host buffers"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        est, desc = cpu_oracle_sample(scene, scene.views[0], args.cpu_tiles)
        cpu = {"value": 1.0 / est, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "P": P, "width": args.width, "height": args.height,
                       "views": len(settings), "parallelism": "replicas" if world > 1 else "1 gpu",
                       "l2": "inputs (708 MB) larger than L2", "mean_instances_K": int(K_avg),
                       "mean_visible": int(V_avg)},
            "roofline": roof, "kernels": kernels, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "clocks": clk}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
