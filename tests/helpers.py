"""Shared test helpers: C-ABI calls with torch-owned buffers, and the
conversion of scenes/views to oracle inputs."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from dmgs_gb300 import _lib
from dmgs_gb300._lib import DmgsGaussians, DmgsGrads, DmgsView, ptr
from oracle import raster as R

MODES = [("shs", "sr"), ("colors", "sr"), ("colors", "cov"), ("shs", "cov")]


def oracle_camera(view, bg=(0.0, 0.0, 0.0), sh_degree=3, scale_modifier=1.0, prefiltered=False):
    return R.Camera(view.width, view.height, view.tanfovx, view.tanfovy, view.viewmatrix,
                    view.projmatrix, view.campos, np.asarray(bg, np.float32),
                    scale_modifier=scale_modifier, sh_degree=sh_degree, prefiltered=prefiltered)


def cov_of_scene(scene, mod=1.0):
    return R.cov3d_from_scale_rot_f32(scene.scales, scene.rotations, mod).astype(np.float32)


def colors_of_scene(scene, seed=7):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 1.0, (scene.P, 3)).astype(np.float32)


def mode_inputs(scene, mode):
    """numpy inputs (means3D, opacities, shs, colors, scales, rotations, cov3D)."""
    col, cv = mode
    shs = scene.shs if col == "shs" else None
    colors = colors_of_scene(scene) if col == "colors" else None
    scales = scene.scales if cv == "sr" else None
    rots = scene.rotations if cv == "sr" else None
    cov = cov_of_scene(scene) if cv == "cov" else None
    return dict(means3D=scene.means3D, opacities=scene.opacities, shs=shs, colors=colors,
                scales=scales, rotations=rots, cov3D=cov)


def _dev(a, device="cuda"):
    if a is None:
        return None
    return torch.as_tensor(np.ascontiguousarray(a)).to(device)


class AbiRun:
    """Forward (and optionally backward) through the C ABI, keeping the
    state buffers for the debug views."""

    def __init__(self, view, inputs, bg=(0.0, 0.0, 0.0), sh_degree=3, scale_modifier=1.0,
                 prefiltered=False, debug=True, device="cuda"):
        self.lib = _lib.load()
        self.device = device
        self.W, self.H = view.width, view.height
        self.t = {k: _dev(v, device) for k, v in inputs.items()}
        self.P = self.t["means3D"].shape[0]
        self.M = self.t["shs"].shape[1] if self.t["shs"] is not None else 0
        self.cam_t = [_dev(np.asarray(bg, np.float32)), _dev(view.viewmatrix), _dev(view.projmatrix),
                      _dev(view.campos)]
        self.view = DmgsView(self.W, self.H, view.tanfovx, view.tanfovy, scale_modifier, sh_degree,
                             int(prefiltered), int(debug), *[ptr(x) for x in self.cam_t])
        t = self.t
        self.g = DmgsGaussians(self.P, self.M, ptr(t["means3D"]), ptr(t["opacities"]), ptr(t["shs"]),
                               ptr(t["colors"]), ptr(t["scales"]), ptr(t["rotations"]), ptr(t["cov3D"]))
        self.stream = torch.cuda.current_stream().cuda_stream

    def forward(self):
        lib = self.lib
        self.geom = torch.empty(lib.dmgs_geom_state_bytes(self.P, self.W, self.H), dtype=torch.uint8,
                                device=self.device)
        self.radii = torch.empty(max(self.P, 1), dtype=torch.int32, device=self.device)
        K = C.c_int64(0)
        _lib.check(lib.dmgs_raster_fwd_geometry(self.view, self.g, self.geom.data_ptr(),
                                                self.geom.numel(), self.radii.data_ptr(),
                                                C.byref(K), self.stream), "fwd_geometry")
        self.K = int(K.value)
        self.bin = torch.empty(lib.dmgs_binning_state_bytes(self.K, self.W, self.H),
                               dtype=torch.uint8, device=self.device)
        self.img = torch.empty(lib.dmgs_image_state_bytes(self.W, self.H), dtype=torch.uint8,
                               device=self.device)
        self.color = torch.empty(3, self.H, self.W, device=self.device)
        _lib.check(lib.dmgs_raster_fwd_render(self.view, self.g, self.geom.data_ptr(),
                                              self.geom.numel(), self.bin.data_ptr(), self.bin.numel(),
                                              self.K, self.img.data_ptr(), self.img.numel(),
                                              self.color.data_ptr(), self.stream), "fwd_render")
        torch.cuda.synchronize()
        return self

    def debug_views(self):
        lib, P, d = self.lib, self.P, self.device
        rect = torch.zeros(max(P, 1), 4, dtype=torch.int32, device=d)
        tiles = torch.zeros(max(P, 1), dtype=torch.int32, device=d)
        depth = torch.zeros(max(P, 1), device=d)
        xy = torch.zeros(max(P, 1), 2, device=d)
        co = torch.zeros(max(P, 1), 4, device=d)
        rgb = torch.zeros(max(P, 1), 3, device=d)
        _lib.check(lib.dmgs_debug_geometry(P, self.W, self.H, self.geom.data_ptr(), self.geom.numel(),
                                           rect.data_ptr(), tiles.data_ptr(), depth.data_ptr(),
                                           xy.data_ptr(), co.data_ptr(), rgb.data_ptr(), self.stream),
                   "debug_geometry")
        gx, gy = (self.W + 15) // 16, (self.H + 15) // 16
        keys = torch.zeros(max(self.K, 1), dtype=torch.int64, device=d)
        vals = torch.zeros(max(self.K, 1), dtype=torch.int32, device=d)
        ranges = torch.zeros(gx * gy, 2, dtype=torch.int32, device=d)
        _lib.check(lib.dmgs_debug_binning(P, self.W, self.H, self.K, self.geom.data_ptr(),
                                          self.geom.numel(), self.bin.data_ptr(), self.bin.numel(),
                                          keys.data_ptr(), vals.data_ptr(), ranges.data_ptr(),
                                          self.stream), "debug_binning")
        fT = torch.zeros(self.H, self.W, device=d)
        nc = torch.zeros(self.H, self.W, dtype=torch.int32, device=d)
        _lib.check(lib.dmgs_debug_image(self.W, self.H, self.img.data_ptr(), self.img.numel(),
                                        fT.data_ptr(), nc.data_ptr(), self.stream), "debug_image")
        torch.cuda.synchronize()
        u32 = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
        return dict(rect=rect.cpu().numpy()[:P], tiles_touched=u32(tiles)[:P],
                    depth=depth.cpu().numpy()[:P], xy=xy.cpu().numpy()[:P],
                    conic_opacity=co.cpu().numpy()[:P], rgb=rgb.cpu().numpy()[:P],
                    keys=keys.cpu().numpy().view(np.uint64)[:self.K], values=u32(vals)[:self.K],
                    ranges=u32(ranges), final_T=fT.cpu().numpy(), n_contrib=u32(nc))

    def backward(self, dL_dimage, f64sum=False):
        """dmgs_raster_bwd (float atomics), or with f64sum=True the FP64-sum
        mode dmgs_raster_bwd_f64sum."""
        lib, P, d = self.lib, self.P, self.device
        z = lambda *s: torch.full(s, float("nan"), device=d)  # noqa: E731  (must be fully written)
        t = self.t
        self.grads = dict(means2D=z(P, 3), colors=z(P, 3), opacities=z(P, 1), means3D=z(P, 3),
                          cov3D=z(P, 6) if t["cov3D"] is not None else None,
                          shs=z(P, self.M, 3) if t["shs"] is not None else None,
                          scales=z(P, 3) if t["scales"] is not None else None,
                          rotations=z(P, 4) if t["rotations"] is not None else None)
        gr = self.grads
        grads = DmgsGrads(ptr(gr["means2D"]), ptr(gr["colors"]), ptr(gr["opacities"]),
                          ptr(gr["means3D"]), ptr(gr["cov3D"]), ptr(gr["shs"]), ptr(gr["scales"]),
                          ptr(gr["rotations"]))
        nbytes = lib.dmgs_bwd_scratch_f64_bytes(P) if f64sum else lib.dmgs_bwd_scratch_bytes(P)
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=d)
        dout = _dev(np.asarray(dL_dimage, np.float32))
        fn = lib.dmgs_raster_bwd_f64sum if f64sum else lib.dmgs_raster_bwd
        _lib.check(fn(self.view, self.g, dout.data_ptr(), self.geom.data_ptr(),
                      self.geom.numel(), self.bin.data_ptr(), self.bin.numel(), self.K,
                      self.img.data_ptr(), self.img.numel(), scratch.data_ptr(), scratch.numel(),
                      grads, self.stream), "raster_bwd")
        torch.cuda.synchronize()
        # the blend adjoint's per-Gaussian 2D gradient records, the first 48 B
        # per Gaussian of the scratch (dL/dndc x, y; dL/dconic a, b, c;
        # dL/dopacity; dL/drgb; 3 unused), for tests of the adjoint alone
        self.records2d = scratch[: P * 48].view(torch.float32).view(P, 12)[:, :9].cpu().numpy()
        return {k: (v.cpu().numpy() if v is not None else None) for k, v in gr.items()}


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / max(den, 1e-30)


# oracle gradient names -> AbiRun gradient names
GRAD_NAMES = {"means3D": "means3D", "means2D": "means2D", "opacities": "opacities",
              "shs": "shs", "colors_precomp": "colors", "scales": "scales",
              "rotations": "rotations", "cov3D_precomp": "cov3D"}


def sampled_tile_lists(geom, gx, tiles):
    """Per tile of `tiles` (row-major tile ids), the visible Gaussians whose
    tile rectangle contains it, in (depth, index) order — the tile lists of
    the reference's (tile, depth) sort, from the oracle's FP32 geometry.
    Returns (lists, union of their Gaussians)."""
    vis = np.nonzero(geom["visible"])[0]
    rect = geom["rect"][vis]
    dbits = geom["depth"][vis].view(np.uint32)
    lists = []
    for t in tiles:
        ty, tx = divmod(int(t), gx)
        m = (rect[:, 0] <= tx) & (tx < rect[:, 2]) & (rect[:, 1] <= ty) & (ty < rect[:, 3])
        ids = vis[m]
        lists.append(ids[np.lexsort((ids, dbits[m]))])
    union = np.unique(np.concatenate(lists)) if lists else np.zeros(0, np.int64)
    return lists, union


def blend_sampled_tiles(width, height, gx, tiles, lists, union, pix, conic, op, rgb, bg, image,
                        seed=3):
    """FP64 oracle blending of the sampled tiles (2D quantities of the
    Gaussians in `union`, in union order) and the comparison with `image`
    ([3,H,W] numpy, the kernel's).  Returns (loss, dL/dimage [3,H,W] float32
    that is N(0,1) on the decidable pixels of the sampled tiles and 0
    elsewhere, the max image error on decidable pixels, the number of those
    pixels)."""
    pos = {int(g): i for i, g in enumerate(union)}
    rng = np.random.default_rng(seed)
    dimg = np.zeros((3, height, width), np.float32)
    loss = 0.0
    err = 0.0
    checked = 0
    bg64 = torch.as_tensor(np.asarray(bg, np.float64))
    for t, ids in zip(tiles, lists):
        ty, tx = divmod(int(t), gx)
        x0, y0 = tx * 16, ty * 16
        x1, y1 = min(x0 + 16, width), min(y0 + 16, height)
        yy, xx = torch.meshgrid(torch.arange(y0, y1, dtype=torch.float64),
                                torch.arange(x0, x1, dtype=torch.float64), indexing="ij")
        pxy = torch.stack([xx.reshape(-1), yy.reshape(-1)], 1)
        g = torch.as_tensor([pos[int(i)] for i in ids], dtype=torch.long)
        out, _, _, amb = R._blend_tile(pxy, pix[g], conic[g], op[g], rgb[g], bg64)
        ok = ~amb.numpy()
        mine = image[:, y0:y1, x0:x1].reshape(3, -1).T
        if ok.any():
            err = max(err, float(np.abs(mine[ok] - out.detach().numpy()[ok]).max()))
        d = rng.standard_normal(out.shape).astype(np.float32) * ok[:, None]
        dimg[:, y0:y1, x0:x1] = d.T.reshape(3, y1 - y0, x1 - x0)
        loss = loss + (out * torch.as_tensor(d, dtype=torch.float64)).sum()
        checked += int(ok.sum())
    return loss, dimg, err, checked
