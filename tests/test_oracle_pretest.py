"""The batched preprocess's per-view pre-test (csrc/preprocess.cu,
preprocess_batched_kernel, phase 1) never culls a (Gaussian, view) pair
that the full FP32 geometry chain keeps visible.

The pre-test's arithmetic is restated here in float32 numpy, with the
kernel's approximate reciprocal and reciprocal square root perturbed by
4 ulp in both directions (their documented error is 2 ulp), and compared with
the oracle's FP32 chain (``oracle.raster.geometry_f32``) on scenes harder
than the GPU tests': coordinates scaled by 1000, wide and narrow fields of
view, scales spanning four decades, Gaussians packed against the near
plane.  The GPU tests check the kernel's own radii against the same oracle
on the large scene; this pins the bound's margins where they are tight."""
import math

import numpy as np
import pytest

from dmgs_gb300.camera import make_view
from dmgs_gb300.scenes import large_scene, random_inside_view
from helpers import oracle_camera
from oracle import raster as R

F = np.float32
ULP4 = F(2.0 ** -21)


def _pretest_keep(means, cov, cam, e_rcp, e_rsq):
    """Candidate mask of the kernel's pre-test for one view."""
    V = np.asarray(cam.viewmatrix, F).reshape(16)
    Pm = np.asarray(cam.projmatrix, F).reshape(16)
    fx, fy = R.focal(cam)
    lx, ly = F(1.3) * F(cam.tanfovx), F(1.3) * F(cam.tanfovy)
    w2 = F(0)
    for j in range(3):
        for i in range(3):
            w2 = F(w2 + V[4 * j + i] * V[4 * j + i])
    kv = F((fx * fx * (F(1) + lx * lx) + fy * fy * (F(1) + ly * ly)) * w2)
    c = cov.astype(F)
    sfro = np.sqrt((c[:, 0] * c[:, 0] + c[:, 3] * c[:, 3] + c[:, 5] * c[:, 5])
                   + F(2) * (c[:, 1] * c[:, 1] + c[:, 2] * c[:, 2] + c[:, 4] * c[:, 4]))
    m = means.astype(F)
    x, y, z = m[:, 0], m[:, 1], m[:, 2]
    vz = ((V[2] * x + V[6] * y) + V[10] * z) + V[14]
    hx = ((Pm[0] * x + Pm[4] * y) + Pm[8] * z) + Pm[12]
    hy = ((Pm[1] * x + Pm[5] * y) + Pm[9] * z) + Pm[13]
    hw = ((Pm[3] * x + Pm[7] * y) + Pm[11] * z) + Pm[15]
    gx, gy = cam.grid
    with np.errstate(all="ignore"):
        pw = (F(1) / (hw + F(1e-7))) * (F(1) + e_rcp)
        px = ((hx * pw + F(1)) * F(cam.width) - F(1)) * F(0.5)
        py = ((hy * pw + F(1)) * F(cam.height) - F(1)) * F(0.5)
        q = (kv * sfro / (vz * vz)) * (F(1) + e_rcp) + F(0.62)
        rb = F(3.0116) * (q * ((F(1) / np.sqrt(q)) * (F(1) + e_rsq))) + F(2)
        ax, ay = F(1e-4) * np.abs(px), F(1e-4) * np.abs(py)
        cull = ((px + rb + ax < F(-1)) | (px - rb - ax > F(16 * gx) + F(2))
                | (py + rb + ay < F(-1)) | (py - rb - ay > F(16 * gy) + F(2)))
        far = ~(vz < F(1e18))
    return (vz > F(0.2)) & (far | ~cull)


def _check(means, scales, rots, views, min_cull=0.0):
    opac = np.full((means.shape[0], 1), 0.5, F)
    cov = R.cov3d_from_scale_rot_f32(scales, rots, F(1.0))
    front = culled = 0
    for view in views:
        cam = oracle_camera(view)
        vis = R.geometry_f32(means, cam, opac, cov3D=cov)["visible"]
        assert vis.any()
        for e_rcp in (-ULP4, ULP4):
            for e_rsq in (-ULP4, ULP4):
                keep = _pretest_keep(means, cov, cam, e_rcp, e_rsq)
                missed = np.nonzero(vis & ~keep)[0]
                assert missed.size == 0, (view.width, view.height, missed[:5])
        m = means.astype(F)
        V = np.asarray(cam.viewmatrix, F).reshape(16)
        inf = (((V[2] * m[:, 0] + V[6] * m[:, 1]) + V[10] * m[:, 2]) + V[14]) > F(0.2)
        front += int(inf.sum())
        culled += int((inf & ~keep).sum())
    assert culled >= min_cull * front, (culled, front)


def test_pretest_on_inside_views_culls_most_pairs_and_misses_none():
    sc = large_scene(P=150_000, seed=11, n_views=1)
    rng = np.random.default_rng(5)
    views = [random_inside_view(rng, 1237, 822) for _ in range(4)]
    _check(sc.means3D, sc.scales, sc.rotations, views, min_cull=0.5)


def test_pretest_with_coordinates_scaled_by_1000():
    sc = large_scene(P=100_000, seed=12, n_views=1)
    k = 1000.0
    rng = np.random.default_rng(6)
    views = []
    for _ in range(3):
        v = random_inside_view(rng, 640, 480)
        eye = np.asarray(v.campos, np.float64) * k
        yaw = rng.uniform(0, 2 * math.pi)
        views.append(make_view(eye, eye + k * np.array([math.cos(yaw), 0.0, math.sin(yaw)]), 640, 480,
                               fovx_deg=60.0, znear=0.01 * k, zfar=100.0 * k))
    _check((sc.means3D * k).astype(F), (sc.scales * k).astype(F), sc.rotations, views, min_cull=0.5)


@pytest.mark.parametrize("fov", [5.0, 120.0])
def test_pretest_at_narrow_and_wide_fields_of_view(fov):
    sc = large_scene(P=100_000, seed=13, n_views=1)
    rng = np.random.default_rng(7)
    views = [random_inside_view(rng, 800, 600, fov_deg=fov) for _ in range(3)]
    _check(sc.means3D, sc.scales, sc.rotations, views)


def test_pretest_with_scales_over_four_decades_and_gaussians_at_the_near_plane():
    rng = np.random.default_rng(8)
    n = 120_000
    eye = np.array([0.0, 0.0, 0.0])
    view = make_view(eye, (0.0, 0.0, 1.0), 512, 384, fovx_deg=70.0)
    # a slab just beyond the 0.2 near cull, wider than the frustum, and a far field
    near = np.stack([rng.uniform(-0.6, 0.6, n // 2), rng.uniform(-0.5, 0.5, n // 2),
                     rng.uniform(0.19, 0.3, n // 2)], 1)
    far = rng.uniform(-30.0, 30.0, (n - n // 2, 3))
    means = np.concatenate([near, far]).astype(F)
    scales = np.exp(rng.uniform(-8.0, 1.0, (n, 3))).astype(F)
    q = rng.standard_normal((n, 4))
    rots = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(F)
    other = make_view((3.0, 1.0, -2.0), (0.0, 0.0, 0.5), 640, 360, fovx_deg=90.0)
    _check(means, scales, rots, [view, other])
