"""The C ABI library: it loads, exports every symbol include/dmgs.h
declares, and rejects invalid arguments on the host (no GPU needed: these
paths return before any CUDA call)."""
import ctypes as C
import os
import re

import pytest

from dmgs_gb300 import _lib
from dmgs_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build()
    return _lib.load()


def _declared():
    src = open(os.path.join(ROOT, "include", "dmgs.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(dmgs_[a-z0-9_]+)\s*\(", src)
    return sorted(set(n for n in names if n != "dmgs_alloc_fn"))


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(names) == bound


def test_sizes_are_consistent(lib):
    header = open(os.path.join(ROOT, "include", "dmgs.h")).read()
    assert f"#define DMGS_ABI_VERSION {_lib.ABI_VERSION}\n" in header
    assert lib.dmgs_abi_version() == _lib.ABI_VERSION
    g1 = lib.dmgs_geom_state_bytes(1000, 256, 256)
    g2 = lib.dmgs_geom_state_bytes(2000, 256, 256)
    assert g2 > g1 and g1 % 256 == 0
    assert lib.dmgs_binning_state_bytes(0, 256, 256) < lib.dmgs_binning_state_bytes(10**6, 256, 256)
    # 12 bytes per instance: the per-tile Gaussian index lists (4 B) and the
    # row lists they are split from (8 B per entry, at most one per instance)
    d = lib.dmgs_binning_state_bytes(2 * 10**6, 64, 64) - lib.dmgs_binning_state_bytes(10**6, 64, 64)
    assert 11.9e6 <= d <= 12.1e6
    assert lib.dmgs_image_state_bytes(1237, 822) >= 1237 * 822 * 8
    assert lib.dmgs_bwd_scratch_bytes(10) >= 480


def _view(**kw):
    v = dict(width=64, height=64, tanfovx=0.5, tanfovy=0.5, scale_modifier=1.0, sh_degree=3,
             prefiltered=0, debug=0, bg=8, viewmatrix=8, projmatrix=8, campos=8)
    v.update(kw)
    return _lib.DmgsView(**v)


def _gauss(**kw):
    g = dict(P=10, M=16, means3D=16, opacities=16, shs=16, colors_precomp=None, scales=16,
             rotations=16, cov3D_precomp=None)
    g.update(kw)
    return _lib.DmgsGaussians(**g)


def _fwd(lib, view, g):
    K = C.c_int64(0)
    return lib.dmgs_raster_fwd_geometry(view, g, 16, 1 << 30, 16, C.byref(K), None)


def test_input_mode_rules(lib):
    assert _fwd(lib, _view(), _gauss(shs=None)) == -1
    assert b"exactly one of either SHs" in lib.dmgs_last_error()
    assert _fwd(lib, _view(), _gauss(colors_precomp=16)) == -1
    assert _fwd(lib, _view(), _gauss(cov3D_precomp=16)) == -1
    assert b"scale/rotation" in lib.dmgs_last_error()
    assert _fwd(lib, _view(), _gauss(scales=None)) == -1
    assert _fwd(lib, _view(), _gauss(M=4)) == -1          # degree 3 needs 16 coefficients
    assert _fwd(lib, _view(), _gauss(rotations=20)) == -1  # misaligned quaternions


def test_view_validation(lib):
    assert _fwd(lib, _view(width=0), _gauss()) == -1
    assert _fwd(lib, _view(sh_degree=4), _gauss()) == -1
    assert _fwd(lib, _view(bg=None), _gauss()) == -1
    assert _fwd(lib, _view(tanfovx=0.0), _gauss()) == -1


def test_state_size_checks(lib):
    K = C.c_int64(0)
    need = lib.dmgs_geom_state_bytes(10, 64, 64)
    assert lib.dmgs_raster_fwd_geometry(_view(), _gauss(), 16, need - 1, 16, C.byref(K), None) == -3
    assert lib.dmgs_raster_fwd_render(_view(), _gauss(), 16, need, 16, 0, 5, 16, 1 << 20, 16, None) == -3
    assert lib.dmgs_raster_fwd_render(_view(), _gauss(), 16, need, 16, 1 << 30, 5, 16, 0, 16, None) == -3
    assert lib.dmgs_bind_fwd(None, None, None, None, None, None) == -1
    assert lib.dmgs_mark_visible(-1, None, None, None, None, None) == -1


def test_flexicubes_tables_match_oracle(lib):
    """The Dual Marching Cubes tables the library derives (host-only call)
    equal the oracle's, which are pinned to the reference's tables."""
    from oracle.flexicubes import derive_tables
    groups = (C.c_uint16 * 1024)()
    nvd = (C.c_uint8 * 256)()
    chk = (C.c_int8 * 1280)()
    assert lib.dmgs_fc_tables(C.addressof(groups), C.addressof(nvd), C.addressof(chk)) == 0
    dmc, num_vd, check = derive_tables()
    for c in range(256):
        assert nvd[c] == num_vd[c]
        for l in range(4):
            edges = [e for e in dmc[c][l] if e != -1]
            assert groups[4 * c + l] == sum(1 << e for e in edges), (c, l)
        got = [chk[5 * c + q] for q in range(5)]
        want = list(check[c])
        want[4] = want[4] - 256 if want[4] > 127 else want[4]  # int8 storage of the complement
        assert got == want, c


def test_flexicubes_rejects_bad_grid(lib):
    g = _lib.DmgsFcGrid(x=8, s=8, rx=0, ry=4, rz=4)
    counts = (C.c_uint32 * 8)()
    assert lib.dmgs_fc_count(C.byref(g), 8, 1 << 20, C.addressof(counts), None) == -1
    g = _lib.DmgsFcGrid(x=8, s=8, rx=4, ry=4, rz=4)
    assert lib.dmgs_fc_count(C.byref(g), 8, 16, C.addressof(counts), None) == -3
    assert lib.dmgs_fc_state_bytes(4, 4, 4) > 4 * 4 * 4 * 5


def test_texture_table_size_matches_oracle(lib):
    """The encoding's level layout (host-only): total table entries."""
    from oracle.texture import per_level_scale, table_entries
    assert lib.dmgs_tex_table_entries(per_level_scale()) == table_entries()
    assert lib.dmgs_tex_table_entries(0.5) == -1


def test_new_entry_points_reject_bad_arguments(lib):
    """Host-side validation of the texture, colour and FlexiCubes entry
    points (each returns before any CUDA call)."""
    tx = _lib.DmgsTexture(table=8, W1=8, W2=8, W3=8, channels=5,
                          aabb=(C.c_float * 6)(-1, -1, -1, 1, 1, 1), per_level_scale=1.447)
    assert lib.dmgs_tex_fwd(C.byref(tx), 10, 8, 8, None) == -1          # channels not 3/12/27/48
    tx.channels = 48
    tx.aabb = (C.c_float * 6)(1, -1, -1, -1, 1, 1)
    assert lib.dmgs_tex_fwd(C.byref(tx), 10, 8, 8, None) == -1          # empty box
    tx.aabb = (C.c_float * 6)(-1, -1, -1, 1, 1, 1)
    assert lib.dmgs_tex_bwd(C.byref(tx), 10, 8, 8, None, None, 8, 8, 8, None, 0, None) == -3
    assert lib.dmgs_tex_bwd(C.byref(tx), 10, 8, 8, None, None, 8, 8, 8, 8, 10 * 128, None) == -3
    assert lib.dmgs_tex_bwd_scratch_bytes(10) == 10 * 128
    assert lib.dmgs_sh_colors_fwd(10, 4, 25, 8, 8, 8, 8, None) == -1     # degree above 3
    assert lib.dmgs_sh_colors_fwd(10, 3, 9, 8, 8, 8, 8, None) == -1      # K < (deg + 1)^2
    assert lib.dmgs_sh_colors_bwd(10, 2, 9, 8, 8, 8, 8, None, None, None) == -1  # no dL/dsh
    g = _lib.DmgsFcGrid(x=8, s=8, rx=4, ry=4, rz=4, beta_stride=5)
    counts = (C.c_uint32 * 8)()
    assert lib.dmgs_fc_count(C.byref(g), 8, 1 << 20, C.addressof(counts), None) == -1  # stride < 12


def test_batch_rejects_unsupported_blend_tuning(lib):
    """dmgs_raster_fwd_batched refuses a blend configuration it has no kernel
    for (pixels per thread, Gaussians per batch, CTA shape) with DMGS_ERR_ARG
    before any device work; the two-tile CTA shapes take 2 or 4 pixels per
    thread and batches of 128 or 256."""
    views = (_lib.DmgsView * 1)(_view())
    out = (C.c_void_p * 1)(16)
    cap = (C.c_int64 * 1)(1 << 20)

    def run(ppt, gpb, shape):
        b = _lib.DmgsBatch(1, views, out, None, cap, ppt, gpb, shape)
        need = lib.dmgs_batch_state_bytes(C.byref(b), 10)
        assert need > 0
        return lib.dmgs_raster_fwd_batched(C.byref(b), C.byref(_gauss()), 256, need, None)

    for ppt, gpb, shape in [(3, 128, 0), (4, 64, 0), (4, 128, 3), (4, 128, -1), (1, 128, 1),
                            (4, 512, 2), (1, 256, 2)]:
        assert run(ppt, gpb, shape) == -1, (ppt, gpb, shape)
        assert b"unsupported blend tuning" in lib.dmgs_last_error()
