"""FlexiCubes isosurface extraction on the GPU (csrc/flexicubes.cu).

Drop-in for the reference's ``geo.flexicubes.FlexiCubes`` as stage 2 uses it
(``scene/gaussian_geo_model_mlp_flex.py:177-181,240-255``): a regular grid
from ``construct_voxel_grid_v2`` and ``__call__(x_nx3, s_n, cube_fx8, res,
beta_fx12, alpha_fx8, gamma_f, training=...)`` returning
``(vertices, faces, L_dev, surf_edges)``, differentiable w.r.t. the vertex
positions, the scalar field and the three raw weight sets.

``FlexiCubesNoAdjacent`` is the drop-in for ``geo.flexicubes_no_adjacent``,
the variant the real-scene stage 2 extracts per view
(``scene/gaussian_geo_model_mlp_flex_colmap.py:298-346``): its
``construct_cubes(vert_mask, res)`` selects the cubes whose corner-0 vertex
is marked (e.g. by :func:`dmgs_gb300.binding.vertex_frustum_mask`) and its
``__call__`` skips the C16/C19 re-check unless ``de_ambiguity=True``.

Not provided (no DMGS caller uses them): the tetrahedral output
(``output_tetmesh=True``), the QEF path (``grad_func``), cube layouts other
than the regular grid or a subset of its cubes in grid order, weights with a
cube subset, and the re-check with a cube subset (the reference's re-check
indexes the whole grid); each raises.
"""
from __future__ import annotations

import ctypes as C
import weakref

import torch

from . import _lib
from ._lib import check, ptr, stream_of

__all__ = ["FlexiCubes", "FlexiCubesNoAdjacent", "flexicubes"]


def _grid(x, s, beta, alpha, gamma, res, training, fused=False, vmask=None, nocheck=False):
    """Kernel arguments.  fused: ``beta`` is the whole [C, 21] weight tensor
    (beta, alpha, gamma = its columns 0-11, 12-19, 20), read in place.
    vmask: uint8 [N] cube subset by corner-0 vertex; nocheck: no C16/C19
    re-check."""
    g = _lib.DmgsFcGrid()
    g.vert_mask = ptr(vmask)
    g.no_ambiguity_check = 1 if nocheck else 0
    g.x, g.s = x.data_ptr(), s.data_ptr()
    if fused:
        g.beta, g.alpha, g.gamma = beta.data_ptr(), beta.data_ptr() + 48, beta.data_ptr() + 80
        g.beta_stride = g.alpha_stride = g.gamma_stride = 21
    else:
        g.beta, g.alpha, g.gamma = ptr(beta), ptr(alpha), ptr(gamma)
    g.rx, g.ry, g.rz = (int(r) for r in res)
    g.training = 1 if training else 0
    return g


def _fused_weights(beta, alpha, gamma, C):
    """The [C, 21] tensor whose column slices 0:12, 12:20 and 20 the three
    weights are (stage 2 slices per_cube_weights this way,
    scene/gaussian_geo_model_mlp_flex.py:246-247), else None."""
    if beta is None or alpha is None or gamma is None:
        return None
    W = beta._base
    if W is None or alpha._base is not W or gamma._base is not W:
        return None
    if W.dtype != torch.float32 or not W.is_contiguous() or tuple(W.shape) != (C, 21):
        return None
    o = W.storage_offset()
    ok = (tuple(beta.shape) == (C, 12) and tuple(alpha.shape) == (C, 8) and tuple(gamma.shape) == (C,)
          and beta.stride() == (21, 1) and alpha.stride() == (21, 1) and gamma.stride() == (21,)
          and beta.storage_offset() == o and alpha.storage_offset() == o + 12
          and gamma.storage_offset() == o + 20)
    return W if ok else None


def _f32(t):
    return None if t is None else t.detach().float().contiguous()


class _FlexiCubesFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, s, beta, alpha, gamma, res, training, fused=False, vmask=None,
                nocheck=False):
        lib = _lib.load()
        dev = x.device
        xs, ss, bs, as_, gs = (_f32(t) for t in (x, s, beta, alpha, gamma))
        grid = _grid(xs, ss, bs, as_, gs, res, training, fused, vmask, nocheck)
        state = torch.empty(lib.dmgs_fc_state_bytes(*grid_res(res)), dtype=torch.uint8, device=dev)
        counts = (C.c_uint32 * 8)()
        stream = stream_of(dev)
        check(lib.dmgs_fc_count(C.byref(grid), state.data_ptr(), state.numel(), C.addressof(counts),
                                stream), "fc_count")
        n_surf, n_vd, n_ent, n_edges, n_quads = (int(counts[k]) for k in range(5))
        work = torch.empty(max(1, lib.dmgs_fc_work_bytes(C.addressof(counts))), dtype=torch.uint8,
                           device=dev)
        nverts = n_vd + (n_quads if training else 0)
        vertices = torch.empty((nverts, 3), dtype=torch.float32, device=dev)
        faces = torch.empty(((4 if training else 2) * n_quads, 3), dtype=torch.int64, device=dev)
        L_dev = torch.empty((n_ent,), dtype=torch.float32, device=dev)
        surf_edges = torch.empty((n_edges, 2), dtype=torch.int64, device=dev)
        if n_surf:
            check(lib.dmgs_fc_emit(C.byref(grid), C.addressof(counts), state.data_ptr(), state.numel(),
                                   work.data_ptr(), work.numel(), vertices.data_ptr(), ptr(faces),
                                   ptr(L_dev), ptr(surf_edges), stream), "fc_emit")
        ctx.res, ctx.training, ctx.counts, ctx.fused = tuple(res), training, bytes(counts), fused
        ctx.nocheck = nocheck
        ctx.has = (beta is not None, alpha is not None, gamma is not None)
        ctx.save_for_backward(xs, ss, bs, as_, gs, state, work, vertices, vmask)
        ctx.mark_non_differentiable(faces, surf_edges)
        return vertices, faces, L_dev, surf_edges

    @staticmethod
    def backward(ctx, dvertices, dfaces, dL_dev, dsurf):
        lib = _lib.load()
        xs, ss, bs, as_, gs, state, work, vertices, vmask = ctx.saved_tensors
        dev = xs.device
        counts = (C.c_uint32 * 8).from_buffer_copy(ctx.counts)
        grid = _grid(xs, ss, bs, as_, gs, ctx.res, ctx.training, ctx.fused, vmask, ctx.nocheck)
        dvert = (dvertices.float().contiguous().clone() if dvertices is not None
                 else torch.zeros_like(vertices))
        dL = dL_dev.float().contiguous() if dL_dev is not None else \
            torch.zeros((int(counts[2]),), dtype=torch.float32, device=dev)
        dx = torch.empty_like(xs)
        ds = torch.empty_like(ss)
        if ctx.fused:  # one [C, 21] gradient, written in place by column
            if not ctx.needs_input_grad[2]:
                db = None
                pb = pa = pg = None
            else:
                db = torch.empty_like(bs)
                pb, pa, pg = db.data_ptr(), db.data_ptr() + 48, db.data_ptr() + 80
            da = dg = None
        else:
            db = torch.empty_like(bs) if ctx.has[0] and ctx.needs_input_grad[2] else None
            da = torch.empty_like(as_) if ctx.has[1] and ctx.needs_input_grad[3] else None
            dg = torch.empty_like(gs) if ctx.has[2] and ctx.needs_input_grad[4] else None
            pb, pa, pg = ptr(db), ptr(da), ptr(dg)
        check(lib.dmgs_fc_bwd(C.byref(grid), C.addressof(counts), state.data_ptr(), state.numel(),
                              work.data_ptr(), work.numel(), ptr(vertices), ptr(dvert), ptr(dL),
                              dx.data_ptr(), ds.data_ptr(), pb, pa, pg, stream_of(dev)), "fc_bwd")
        return dx, ds, db, da, dg, None, None, None, None, None


def grid_res(res):
    if isinstance(res, int):
        return (res, res, res)
    r = tuple(int(v) for v in res)
    if len(r) != 3 or min(r) <= 0:
        raise ValueError(f"grid resolution must be 3 positive integers, got {res}")
    return r


def flexicubes(x_nx3, s_n, res, beta_fx12=None, alpha_fx8=None, gamma_f=None, training=False,
               vert_mask=None, de_ambiguity=True):
    """FlexiCubes triangle extraction on the regular grid of ``res``; see
    ``FlexiCubes.__call__``.  vert_mask (bool/uint8 [N]): only the cubes whose
    corner-0 vertex is marked take part (no weights then); de_ambiguity:
    the C16/C19 re-check (not with a cube subset)."""
    res = grid_res(res)
    N = (res[0] + 1) * (res[1] + 1) * (res[2] + 1)
    Cn = res[0] * res[1] * res[2]
    if not x_nx3.is_cuda:
        raise RuntimeError("flexicubes: inputs must be CUDA tensors (no CPU path)")
    if tuple(x_nx3.shape) != (N, 3) or tuple(s_n.reshape(-1).shape) != (N,):
        raise ValueError(f"flexicubes: x [{N},3] and s [{N}] expected for grid {res}")
    for name, t, shp in (("beta_fx12", beta_fx12, (Cn, 12)), ("alpha_fx8", alpha_fx8, (Cn, 8)),
                         ("gamma_f", gamma_f, (Cn,))):
        if t is not None and tuple(t.shape) != shp:
            raise ValueError(f"flexicubes: {name} must be {list(shp)}, got {list(t.shape)}")
    vm = None
    if vert_mask is not None:
        if beta_fx12 is not None or alpha_fx8 is not None or gamma_f is not None:
            raise NotImplementedError("flexicubes: per-cube weights with a cube subset are not provided")
        if de_ambiguity:
            raise NotImplementedError("flexicubes: the C16/C19 re-check needs the whole grid "
                                      "(the reference's re-check indexes every cube)")
        if tuple(vert_mask.reshape(-1).shape) != (N,):
            raise ValueError(f"flexicubes: vert_mask must hold {N} values")
        vm = vert_mask.reshape(-1).to(device=x_nx3.device, dtype=torch.uint8).contiguous()
    nocheck = not de_ambiguity
    W = _fused_weights(beta_fx12, alpha_fx8, gamma_f, Cn)
    if W is not None:  # the three weights are column slices of one tensor: read it in place
        v, f, L, se = _FlexiCubesFn.apply(x_nx3, s_n.reshape(-1), W, None, None, res,
                                          bool(training), True, vm, nocheck)
    else:
        v, f, L, se = _FlexiCubesFn.apply(x_nx3, s_n.reshape(-1), beta_fx12, alpha_fx8,
                                          gamma_f, res, bool(training), False, vm, nocheck)
    if v.shape[0] == 0 and f.shape[0] == 0 and se.shape[0] == 0:
        return v, f, L, None   # the reference's result for a grid without surface
    return v, f, L, se


class FlexiCubes:
    """GPU FlexiCubes with the reference class's interface
    (``geo/flexicubes.py:16-180``) for the regular-grid triangle path."""

    def __init__(self, device="cuda", qef_reg_scale=1e-3, weight_scale=0.99):
        if abs(weight_scale - 0.99) > 1e-12:
            raise NotImplementedError("FlexiCubes: only weight_scale=0.99 (the reference default)")
        self.device = device
        self.qef_reg_scale = qef_reg_scale
        self.weight_scale = weight_scale
        self._regular = ()

    def construct_voxel_grid_v2(self, res, xyz_min=None, xyz_max=None):
        """Vertices [(rx+1)(ry+1)(rz+1), 3] on linspace axes and the corner
        indices of each cube [rx ry rz, 8], both in (i, j, k) order
        (``geo/flexicubes.py:133-157``)."""
        res = grid_res(res)
        lo = [-0.5] * 3 if xyz_min is None else [float(v) for v in xyz_min]
        hi = [0.5] * 3 if xyz_max is None else [float(v) for v in xyz_max]
        axes = [torch.linspace(lo[d], hi[d], res[d] + 1, device=self.device) for d in range(3)]
        verts = torch.stack(torch.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
        return verts, self._cubes(res)

    def _cubes(self, res):
        rx, ry, rz = res
        dev = self.device
        i = torch.arange(rx, device=dev).view(-1, 1, 1)
        j = torch.arange(ry, device=dev).view(1, -1, 1)
        k = torch.arange(rz, device=dev).view(1, 1, -1)
        base = ((i * (ry + 1) + j) * (rz + 1) + k).reshape(-1, 1)
        n = torch.arange(8, device=dev)
        off = (n & 1) * (ry + 1) * (rz + 1) + ((n >> 1) & 1) * (rz + 1) + ((n >> 2) & 1)
        return base + off.view(1, 8)   # int64, as the reference's sum over int32 gives

    @staticmethod
    def _cached(cache, cube_fx8, res):
        """(hit, value) for the cube tensor remembered in `cache` — the same
        tensor object (a weak reference, so a new tensor at a recycled
        address never matches), unmodified, for the same resolution."""
        if cache and cache[0]() is cube_fx8 and cache[1] == cube_fx8._version and cache[2] == res:
            return True, cache[3]
        return False, None

    def _check_regular(self, cube_fx8, res):
        if self._cached(self._regular, cube_fx8, res)[0]:
            return
        ok = tuple(cube_fx8.shape) == (res[0] * res[1] * res[2], 8) and bool(
            torch.equal(cube_fx8.to(torch.int64), self._cubes(res).to(cube_fx8.device).to(torch.int64)))
        if not ok:
            raise NotImplementedError("FlexiCubes: cube_fx8 must be the regular grid of "
                                      "construct_voxel_grid_v2 for this resolution")
        self._regular = (weakref.ref(cube_fx8), cube_fx8._version, res, True)

    def __call__(self, x_nx3, s_n, cube_fx8, res, beta_fx12=None, alpha_fx8=None, gamma_f=None,
                 training=False, output_tetmesh=False, grad_func=None):
        if output_tetmesh:
            raise NotImplementedError("FlexiCubes: tetrahedral output is not provided")
        if grad_func is not None:
            raise NotImplementedError("FlexiCubes: the grad_func (QEF) path is not provided")
        res = grid_res(res)
        self._check_regular(cube_fx8, res)
        return flexicubes(x_nx3, s_n, res, beta_fx12, alpha_fx8, gamma_f, training)


class FlexiCubesNoAdjacent(FlexiCubes):
    """GPU drop-in for the reference's ``geo.flexicubes_no_adjacent.FlexiCubes``
    (the per-view extraction of the real-scene stage 2,
    ``scene/gaussian_geo_model_mlp_flex_colmap.py:298-346``): the grid of
    ``construct_voxel_grid_vert_only``, cube subsets from ``construct_cubes``
    and no C16/C19 re-check by default (``de_ambiguity=False``)."""

    def __init__(self, device="cuda", qef_reg_scale=1e-3, weight_scale=0.99):
        super().__init__(device, qef_reg_scale, weight_scale)
        self._subsets = ()

    def construct_voxel_grid_vert_only(self, res, xyz_min=None, xyz_max=None):
        """Grid vertices [(rx+1)(ry+1)(rz+1), 3] in (i, j, k) order
        (geo/flexicubes_no_adjacent.py:100-127)."""
        return self.construct_voxel_grid_v2(res, xyz_min, xyz_max)[0]

    def construct_cubes(self, vert_mask, res):
        """Corner indices [n, 8] of the cubes whose corner-0 vertex is marked
        and lies inside the grid, in grid order
        (geo/flexicubes_no_adjacent.py:129-145).  The mask is remembered for
        the extraction, which then runs on the subset directly."""
        res = grid_res(res)
        m = vert_mask.reshape(res[0] + 1, res[1] + 1, res[2] + 1).bool()
        inner = m[:res[0], :res[1], :res[2]]
        cubes = self._cubes(res).to(vert_mask.device)[inner.reshape(-1)]
        full = torch.zeros_like(m)
        full[:res[0], :res[1], :res[2]] = inner
        self._subsets = (weakref.ref(cubes), cubes._version, res, full.reshape(-1).to(torch.uint8))
        return cubes

    def _subset_mask(self, cube_fx8, res):
        """The vertex mask of a cube list that is a subset of the grid's cubes
        in grid order, or None for the whole grid."""
        hit, mask = self._cached(self._subsets, cube_fx8, res)
        if hit:
            return mask
        if tuple(cube_fx8.shape) == (res[0] * res[1] * res[2], 8):
            self._check_regular(cube_fx8, res)
            return None
        c = cube_fx8.to(torch.int64)
        base = c[:, 0]
        n = torch.arange(8, device=c.device)
        off = (n & 1) * (res[1] + 1) * (res[2] + 1) + ((n >> 1) & 1) * (res[2] + 1) + ((n >> 2) & 1)
        N = (res[0] + 1) * (res[1] + 1) * (res[2] + 1)
        sy, sx = res[2] + 1, (res[1] + 1) * (res[2] + 1)
        ok = (c.dim() == 2 and c.shape[1] == 8 and bool((c == base.view(-1, 1) + off).all())
              and bool((base[1:] > base[:-1]).all()) and bool((base >= 0).all())
              and bool((base < N).all()) and bool(((base // sx) < res[0]).all())
              and bool((((base // sy) % (res[1] + 1)) < res[1]).all())
              and bool(((base % sy) < res[2]).all()))
        if not ok:
            raise NotImplementedError("FlexiCubesNoAdjacent: cube_fx8 must be cubes of the regular "
                                      "grid in grid order (construct_cubes)")
        mask = torch.zeros(N, dtype=torch.uint8, device=c.device)
        mask[base] = 1
        self._subsets = (weakref.ref(cube_fx8), cube_fx8._version, res, mask)
        return mask

    def __call__(self, x_nx3, s_n, cube_fx8, res, beta_fx12=None, alpha_fx8=None, gamma_f=None,
                 training=False, output_tetmesh=False, grad_func=None, de_ambiguity=False):
        if output_tetmesh:
            raise NotImplementedError("FlexiCubes: tetrahedral output is not provided")
        if grad_func is not None:
            raise NotImplementedError("FlexiCubes: the grad_func (QEF) path is not provided")
        res = grid_res(res)
        mask = self._subset_mask(cube_fx8, res)
        if mask is None:
            return flexicubes(x_nx3, s_n, res, beta_fx12, alpha_fx8, gamma_f, training,
                              de_ambiguity=de_ambiguity)
        if cube_fx8.shape[0] == 0:
            return (x_nx3.new_zeros((0, 3)), torch.zeros((0, 3), dtype=torch.long, device=x_nx3.device),
                    x_nx3.new_zeros((0,)), None)
        return flexicubes(x_nx3, s_n, res, beta_fx12, alpha_fx8, gamma_f, training,
                          vert_mask=mask, de_ambiguity=de_ambiguity)
