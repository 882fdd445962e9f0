"""ctypes binding of libdmgs_gb300.so (the C ABI declared in include/dmgs.h).

The library is loaded once, after torch (which brings the CUDA runtime).
There is no fallback: a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import torch  # noqa: F401  (loads libcudart before the extension)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdmgs_gb300.so")
ABI_VERSION = 8  # DMGS_ABI_VERSION of include/dmgs.h that SIGNATURES and the structs follow

c_float_p = C.POINTER(C.c_float)
vp = C.c_void_p


class DmgsView(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("tanfovx", C.c_float), ("tanfovy", C.c_float),
                ("scale_modifier", C.c_float), ("sh_degree", C.c_int32),
                ("prefiltered", C.c_int32), ("debug", C.c_int32),
                ("bg", vp), ("viewmatrix", vp), ("projmatrix", vp), ("campos", vp)]


class DmgsGaussians(C.Structure):
    _fields_ = [("P", C.c_int32), ("M", C.c_int32),
                ("means3D", vp), ("opacities", vp), ("shs", vp), ("colors_precomp", vp),
                ("scales", vp), ("rotations", vp), ("cov3D_precomp", vp)]


class DmgsGrads(C.Structure):
    _fields_ = [("dL_dmeans2D", vp), ("dL_dcolors", vp), ("dL_dopacity", vp),
                ("dL_dmeans3D", vp), ("dL_dcov3D", vp), ("dL_dsh", vp),
                ("dL_dscales", vp), ("dL_drotations", vp)]


class DmgsFaceBinding(C.Structure):
    _fields_ = [("F", C.c_int32), ("V", C.c_int32), ("G", C.c_int32),
                ("bc_per_gaussian", C.c_int32), ("adaptive_cov", C.c_int32),
                ("rad_base", C.c_float), ("z_scale", C.c_float), ("max_scale", C.c_float),
                ("verts", vp), ("faces", vp), ("bc", vp), ("scale_factor", vp)]


class DmgsFaceBinding3(C.Structure):
    _fields_ = [("F", C.c_int32), ("V", C.c_int32), ("G", C.c_int32), ("thin_z", C.c_float),
                ("verts", vp), ("faces", vp), ("bc", vp), ("scaling2d", vp), ("rotation2d", vp)]


class DmgsFcGrid(C.Structure):
    _fields_ = [("x", vp), ("s", vp), ("beta", vp), ("alpha", vp), ("gamma", vp),
                ("rx", C.c_int32), ("ry", C.c_int32), ("rz", C.c_int32), ("training", C.c_int32),
                ("beta_stride", C.c_int32), ("alpha_stride", C.c_int32), ("gamma_stride", C.c_int32),
                ("vert_mask", vp), ("no_ambiguity_check", C.c_int32)]


class DmgsTexture(C.Structure):
    _fields_ = [("table", vp), ("W1", vp), ("W2", vp), ("W3", vp), ("channels", C.c_int32),
                ("aabb", C.c_float * 6), ("per_level_scale", C.c_float)]


class DmgsBatch(C.Structure):
    _fields_ = [("nviews", C.c_int32), ("views", C.POINTER(DmgsView)),
                ("out_color", C.POINTER(vp)), ("radii", C.POINTER(vp)),
                ("capacity", C.POINTER(C.c_int64)), ("pixels_per_thread", C.c_int32),
                ("gaussians_per_batch", C.c_int32), ("tile_shape", C.c_int32)]


DMGS_ERRORS = {-1: "DMGS_ERR_ARG", -2: "DMGS_ERR_CUDA", -3: "DMGS_ERR_STATE",
               -4: "DMGS_ERR_PREFILTER", -5: "DMGS_ERR_OVERFLOW", -6: "DMGS_ERR_DEVICE"}

# (name, restype, argtypes) for every symbol of include/dmgs.h
SIGNATURES = [
    ("dmgs_geom_state_bytes", C.c_size_t, [C.c_int32, C.c_int32, C.c_int32]),
    ("dmgs_binning_state_bytes", C.c_size_t, [C.c_int64, C.c_int32, C.c_int32]),
    ("dmgs_image_state_bytes", C.c_size_t, [C.c_int32, C.c_int32]),
    ("dmgs_bwd_scratch_bytes", C.c_size_t, [C.c_int32]),
    ("dmgs_raster_fwd_geometry", C.c_int, [C.POINTER(DmgsView), C.POINTER(DmgsGaussians), vp,
                                           C.c_size_t, vp, C.POINTER(C.c_int64), vp]),
    ("dmgs_raster_fwd_render", C.c_int, [C.POINTER(DmgsView), C.POINTER(DmgsGaussians), vp,
                                         C.c_size_t, vp, C.c_size_t, C.c_int64, vp, C.c_size_t,
                                         vp, vp]),
    ("dmgs_raster_fwd", C.c_int, [C.POINTER(DmgsView), C.POINTER(DmgsGaussians), vp, vp, vp,
                                  vp, C.POINTER(C.c_int64), vp]),
    ("dmgs_raster_bwd", C.c_int, [C.POINTER(DmgsView), C.POINTER(DmgsGaussians), vp, vp,
                                  C.c_size_t, vp, C.c_size_t, C.c_int64, vp, C.c_size_t, vp,
                                  C.c_size_t, C.POINTER(DmgsGrads), vp]),
    ("dmgs_bwd_scratch_f64_bytes", C.c_size_t, [C.c_int32]),
    ("dmgs_raster_bwd_f64sum", C.c_int, [C.POINTER(DmgsView), C.POINTER(DmgsGaussians), vp, vp,
                                         C.c_size_t, vp, C.c_size_t, C.c_int64, vp, C.c_size_t,
                                         vp, C.c_size_t, C.POINTER(DmgsGrads), vp]),
    ("dmgs_raster_bwd_noalloc", C.c_int, [C.POINTER(DmgsView), C.POINTER(DmgsGaussians), vp,
                                          vp, C.c_size_t, vp, C.c_size_t, C.c_int64, vp,
                                          C.c_size_t, C.POINTER(DmgsGrads), vp]),
    ("dmgs_batch_state_bytes", C.c_size_t, [C.POINTER(DmgsBatch), C.c_int32]),
    ("dmgs_raster_fwd_batched", C.c_int, [C.POINTER(DmgsBatch), C.POINTER(DmgsGaussians), vp,
                                          C.c_size_t, vp]),
    ("dmgs_raster_bwd_batched", C.c_int, [C.POINTER(DmgsBatch), C.POINTER(DmgsGaussians),
                                          C.POINTER(vp), vp, C.c_size_t, C.POINTER(DmgsGrads),
                                          C.POINTER(vp), vp, vp, vp]),
    ("dmgs_batch_counters", C.c_int, [C.POINTER(DmgsBatch), C.c_int32, vp, C.c_size_t,
                                      C.POINTER(C.c_uint32), vp]),
    ("dmgs_batch_status", C.c_int, [C.POINTER(DmgsBatch), C.c_int32, vp, C.c_size_t,
                                    C.POINTER(C.c_int64), vp]),
    ("dmgs_multi_view_state_bytes", C.c_size_t, [C.POINTER(DmgsView), C.POINTER(DmgsGaussians),
                                                 C.c_int64]),
    ("dmgs_render_multi", C.c_int, [C.POINTER(DmgsBatch), C.POINTER(DmgsGaussians), C.POINTER(vp),
                                    C.POINTER(C.c_size_t), vp, vp]),
    ("dmgs_multi_status_async", C.c_int, [C.POINTER(DmgsBatch), C.POINTER(DmgsGaussians),
                                          C.POINTER(vp), C.POINTER(C.c_size_t), vp, vp]),
    ("dmgs_vertex_frustum_mask", C.c_int, [vp, C.c_int32, vp, C.c_float, C.c_int32, C.c_int32, vp, vp,
                                           vp]),
    ("dmgs_face_cull_scratch_bytes", C.c_size_t, [C.c_int32]),
    ("dmgs_face_cull", C.c_int, [vp, C.c_int32, vp, C.c_int32, vp, vp, vp, vp, vp, C.c_size_t,
                                 vp]),
    ("dmgs_fc_tables", C.c_int, [vp, vp, vp]),
    ("dmgs_fc_state_bytes", C.c_size_t, [C.c_int32, C.c_int32, C.c_int32]),
    ("dmgs_fc_work_bytes", C.c_size_t, [vp]),
    ("dmgs_fc_count", C.c_int, [C.POINTER(DmgsFcGrid), vp, C.c_size_t, vp, vp]),
    ("dmgs_fc_emit", C.c_int, [C.POINTER(DmgsFcGrid), vp, vp, C.c_size_t, vp, C.c_size_t, vp, vp,
                               vp, vp, vp]),
    ("dmgs_fc_bwd", C.c_int, [C.POINTER(DmgsFcGrid), vp, vp, C.c_size_t, vp, C.c_size_t, vp, vp,
                              vp, vp, vp, vp, vp, vp, vp]),
    ("dmgs_sh_colors_fwd", C.c_int, [C.c_int32, C.c_int32, C.c_int32, vp, vp, vp, vp, vp]),
    ("dmgs_sh_colors_bwd", C.c_int, [C.c_int32, C.c_int32, C.c_int32, vp, vp, vp, vp, vp, vp, vp]),
    ("dmgs_tex_table_entries", C.c_int64, [C.c_float]),
    ("dmgs_tex_fwd", C.c_int, [C.POINTER(DmgsTexture), C.c_int64, vp, vp, vp]),
    ("dmgs_tex_fwd_enc", C.c_int, [C.POINTER(DmgsTexture), C.c_int64, vp, vp, vp, vp]),
    ("dmgs_tex_bwd_scratch_bytes", C.c_size_t, [C.c_int64]),
    ("dmgs_tex_bwd", C.c_int, [C.POINTER(DmgsTexture), C.c_int64, vp, vp, vp, vp, vp, vp, vp, vp,
                               C.c_size_t, vp]),
    ("dmgs_tex_bwd_enc", C.c_int, [C.POINTER(DmgsTexture), C.c_int64, vp, vp, vp, vp, vp, vp, vp,
                                   vp, vp, C.c_size_t, vp]),
    ("dmgs_l1_ssim_scratch_bytes", C.c_size_t, [C.c_int32, C.c_int32, C.c_int32]),
    ("dmgs_l1_ssim", C.c_int, [vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_float, vp, vp, vp,
                               C.c_size_t, vp]),
    ("dmgs_mark_visible", C.c_int, [C.c_int32, vp, vp, vp, vp, vp]),
    ("dmgs_debug_geometry", C.c_int, [C.c_int32, C.c_int32, C.c_int32, vp, C.c_size_t, vp, vp,
                                      vp, vp, vp, vp, vp]),
    ("dmgs_debug_binning", C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int64, vp,
                                     C.c_size_t, vp, C.c_size_t, vp, vp, vp, vp]),
    ("dmgs_debug_image", C.c_int, [C.c_int32, C.c_int32, vp, C.c_size_t, vp, vp, vp]),
    ("dmgs_bind_fwd", C.c_int, [C.POINTER(DmgsFaceBinding), vp, vp, vp, vp, vp]),
    ("dmgs_bind_bwd", C.c_int, [C.POINTER(DmgsFaceBinding), vp, vp, vp, vp, vp]),
    ("dmgs_bind3_fwd", C.c_int, [C.POINTER(DmgsFaceBinding3), vp, vp, vp, vp]),
    ("dmgs_bind3_bwd", C.c_int, [C.POINTER(DmgsFaceBinding3), vp, vp, vp, vp, vp, vp, vp]),
    ("dmgs_timing_enable", C.c_int, [C.c_int32]),
    ("dmgs_kernel_launches", C.c_int64, []),
    ("dmgs_timing_collect", C.c_int, [C.POINTER(C.c_int32), C.POINTER(C.c_char_p),
                                      C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ("dmgs_last_error", C.c_char_p, []),
    ("dmgs_abi_version", C.c_int32, []),
]

_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Load the library (once) and declare every signature."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"{p} is missing: build it with `python -m dmgs_gb300.build` "
                "(or __graft_entry__.build()); the rasteriser has no CPU fallback")
        lib = C.CDLL(p)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.dmgs_abi_version() != ABI_VERSION:
            raise RuntimeError(f"{p} has ABI version {lib.dmgs_abi_version()}, this package expects "
                               f"{ABI_VERSION}: rebuild it with `python -m dmgs_gb300.build`")
        _lib = lib
        return lib


class DmgsError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {DMGS_ERRORS.get(code, code)}: {msg}")
        self.code = code


def check(code: int, where: str):
    if code != 0:
        msg = load().dmgs_last_error()
        raise DmgsError(code, where, msg.decode() if msg else "")


def ptr(t) -> int | None:
    """Device address of a tensor (None for None / empty)."""
    if t is None:
        return None
    if t.numel() == 0:
        return None
    return t.data_ptr()


def stream_of(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def timing_enable(on: bool):
    load().dmgs_timing_enable(1 if on else 0)


def timing_collect():
    """{kernel name: (total_ms, launches)} since the last collect."""
    lib = load()
    cap = 64
    n = C.c_int32(cap)
    names = (C.c_char_p * cap)()
    ms = (C.c_double * cap)()
    cnt = (C.c_int64 * cap)()
    lib.dmgs_timing_collect(C.byref(n), names, ms, cnt)
    return {names[i].decode(): (ms[i], cnt[i]) for i in range(n.value)}
