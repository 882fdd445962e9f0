"""GPU parity of the rasteriser (C ABI) against the CPU oracle.

Bars: integer outputs (radii, tile rectangles, tiles_touched, depth keys,
sorted keys/values, tile ranges, n_contrib) bit-exact; images within
2e-4 max-abs on pixels whose value FP32 can decide (the oracle flags the
rest); gradients within 1e-3 relative L2 per input.
"""
import numpy as np
import pytest
import torch

from dmgs_gb300.scenes import small_scene
from helpers import GRAD_NAMES, MODES, AbiRun, mode_inputs, oracle_camera, rel_l2
from oracle import raster as R

pytestmark = pytest.mark.gpu

IMG_TOL = 2e-4
GRAD_TOL = 1e-3


def _check_integer_outputs(run, ref, cam):
    dv = run.debug_views()
    g = ref.geom
    vis = g["visible"]
    np.testing.assert_array_equal(run.radii.cpu().numpy()[:run.P], ref.radii)
    rect_ref = np.where(vis[:, None], g["rect"], 0)
    np.testing.assert_array_equal(dv["rect"], rect_ref)
    np.testing.assert_array_equal(dv["tiles_touched"], g["tiles_touched"])
    np.testing.assert_array_equal(dv["depth"][vis].view(np.uint32), g["depth"][vis].view(np.uint32))
    assert run.K == ref.num_rendered
    np.testing.assert_array_equal(dv["keys"], ref.keys)
    np.testing.assert_array_equal(dv["values"], ref.values)
    np.testing.assert_array_equal(dv["ranges"], ref.ranges)
    return dv


@pytest.mark.parametrize("mode", MODES, ids=["-".join(m) for m in MODES])
def test_cfg1_forward_backward(mode):
    """10k Gaussians, 256x256: the plain-rasteriser workload, all four input modes."""
    sc = small_scene()
    view = sc.views[0]
    inp = mode_inputs(sc, mode)
    cam = oracle_camera(view)
    ref = R.render(cam, inp["means3D"], inp["opacities"], shs=inp["shs"], colors=inp["colors"],
                   scales=inp["scales"], rotations=inp["rotations"], cov3D=inp["cov3D"])
    run = AbiRun(view, inp).forward()
    dv = _check_integer_outputs(run, ref, cam)
    img = run.color.cpu().numpy()
    ok = ~ref.ambiguous
    err = np.abs(img - ref.image)[:, ok].max()
    assert err <= IMG_TOL, err
    np.testing.assert_array_equal(dv["n_contrib"][ok], ref.n_contrib[ok])
    assert np.abs(dv["final_T"] - ref.final_T)[ok].max() <= IMG_TOL

    dimg = np.random.default_rng(0).standard_normal(img.shape).astype(np.float32)
    gk = run.backward(dimg)
    go = ref.backward(dimg)
    for name, gref in go.items():
        mine = gk[GRAD_NAMES[name]]
        assert np.isfinite(mine).all(), name
        e = rel_l2(mine, gref)
        assert e <= GRAD_TOL, (name, e)


def test_background_and_scale_modifier():
    sc = small_scene(P=3000, width=200, height=120, seed=3)
    view = sc.views[0]
    inp = mode_inputs(sc, ("shs", "sr"))
    bg = (0.2, 0.5, 1.0)
    cam = oracle_camera(view, bg=bg, scale_modifier=1.7)
    ref = R.render(cam, inp["means3D"], inp["opacities"], shs=inp["shs"], scales=inp["scales"],
                   rotations=inp["rotations"])
    run = AbiRun(view, inp, bg=bg, scale_modifier=1.7).forward()
    _check_integer_outputs(run, ref, cam)
    ok = ~ref.ambiguous
    assert np.abs(run.color.cpu().numpy() - ref.image)[:, ok].max() <= IMG_TOL
    dimg = np.random.default_rng(1).standard_normal((3, 120, 200)).astype(np.float32)
    gk, go = run.backward(dimg), ref.backward(dimg)
    for name, gref in go.items():
        assert rel_l2(gk[GRAD_NAMES[name]], gref) <= GRAD_TOL, name


@pytest.mark.parametrize("deg", [0, 1, 2])
def test_lower_sh_degrees(deg):
    sc = small_scene(P=2000, width=96, height=80, seed=4)
    view = sc.views[0]
    inp = mode_inputs(sc, ("shs", "sr"))
    cam = oracle_camera(view, sh_degree=deg)
    ref = R.render(cam, inp["means3D"], inp["opacities"], shs=inp["shs"], scales=inp["scales"],
                   rotations=inp["rotations"])
    run = AbiRun(view, inp, sh_degree=deg).forward()
    ok = ~ref.ambiguous
    assert np.abs(run.color.cpu().numpy() - ref.image)[:, ok].max() <= IMG_TOL
    dimg = np.random.default_rng(2).standard_normal((3, 80, 96)).astype(np.float32)
    gk, go = run.backward(dimg), ref.backward(dimg)
    for name, gref in go.items():
        assert rel_l2(gk[GRAD_NAMES[name]], gref) <= GRAD_TOL, name
    # coefficients above the active degree get zero gradient
    assert np.all(gk["shs"][:, (deg + 1) ** 2:, :] == 0)


def test_empty_and_all_culled():
    sc = small_scene(P=500, width=64, height=64, seed=5)
    view = sc.views[0]
    # everything behind the camera: move the means far behind
    inp = mode_inputs(sc, ("colors", "sr"))
    eye = view.campos.astype(np.float64)
    inp["means3D"] = (eye + 3.0 * (eye / np.linalg.norm(eye))
                      + 0.1 * inp["means3D"]).astype(np.float32)
    run = AbiRun(view, inp, bg=(0.3, 0.2, 0.1)).forward()
    assert run.K == 0
    assert (run.radii.cpu().numpy()[:run.P] == 0).all()
    img = run.color.cpu().numpy()
    np.testing.assert_allclose(img, np.broadcast_to(np.array([0.3, 0.2, 0.1], np.float32)[:, None, None], img.shape))
    gk = run.backward(np.ones((3, 64, 64), np.float32))
    for k, v in gk.items():
        if v is not None:
            assert (v == 0).all(), k
    # P == 0
    empty = {k: (None if v is None else v[:0]) for k, v in mode_inputs(sc, ("colors", "sr")).items()}
    run0 = AbiRun(view, empty, bg=(1.0, 1.0, 1.0)).forward()
    assert run0.K == 0
    assert np.all(run0.color.cpu().numpy() == 1.0)


def test_ragged_image_and_long_tile_lists():
    """Image size not a multiple of 16, and > 4096 Gaussians in single tiles
    (the segment sort's chunk-and-merge path)."""
    rng = np.random.default_rng(11)
    P = 12000
    sc = small_scene(P=P, width=37, height=21, seed=6)
    # concentrate everything in a small volume in front of the camera
    view = sc.views[0]
    eye = view.campos.astype(np.float64)
    fwd = -eye / np.linalg.norm(eye)
    sc.means3D[:] = (eye + 2.0 * fwd + rng.normal(0, 0.02, (P, 3))).astype(np.float32)
    sc.scales[:] = np.exp(rng.uniform(-5, -3.5, (P, 3))).astype(np.float32)
    sc.opacities[:] = 0.05
    inp = mode_inputs(sc, ("shs", "sr"))
    cam = oracle_camera(view)
    ref = R.render(cam, inp["means3D"], inp["opacities"], shs=inp["shs"], scales=inp["scales"],
                   rotations=inp["rotations"])
    assert (ref.ranges[:, 1] - ref.ranges[:, 0]).max() > 4096
    run = AbiRun(view, inp).forward()
    _check_integer_outputs(run, ref, cam)
    ok = ~ref.ambiguous
    assert np.abs(run.color.cpu().numpy() - ref.image)[:, ok].max() <= IMG_TOL
    dimg = rng.standard_normal((3, 21, 37)).astype(np.float32)
    gk, go = run.backward(dimg), ref.backward(dimg)
    for name, gref in go.items():
        assert rel_l2(gk[GRAD_NAMES[name]], gref) <= GRAD_TOL, name


def test_wide_image_lists_bit_exact():
    """An image 2,200 pixels wide (138 tiles per row: the emission's masks
    span five 32-tile chunks, and one row of tiles holds more instances than
    a staging sub-pass): sorted keys, values and tile ranges equal the
    oracle's, and the image matches."""
    sc = small_scene(P=20000, width=2200, height=400, fov_deg=60.0, seed=12)
    view = sc.views[0]
    inp = mode_inputs(sc, ("shs", "sr"))
    cam = oracle_camera(view)
    ref = R.render(cam, inp["means3D"], inp["opacities"], shs=inp["shs"], scales=inp["scales"],
                   rotations=inp["rotations"])
    assert (2200 + 15) // 16 > 128 and ref.num_rendered > 100_000
    run = AbiRun(view, inp).forward()
    _check_integer_outputs(run, ref, cam)
    ok = ~ref.ambiguous
    assert np.abs(run.color.cpu().numpy() - ref.image)[:, ok].max() <= IMG_TOL


def test_large_footprints_and_clamped_jacobian():
    """Gaussians close to the camera (hundreds of tiles each) and beyond the
    1.3x field-of-view clamp."""
    rng = np.random.default_rng(12)
    sc = small_scene(P=300, width=160, height=96, seed=7)
    view = sc.views[0]
    eye = view.campos.astype(np.float64)
    fwd = -eye / np.linalg.norm(eye)
    side = np.cross(fwd, [0, 1, 0]); side /= np.linalg.norm(side)
    d = rng.uniform(0.5, 1.5, (300, 1))
    lat = rng.uniform(-1.2, 1.2, (300, 1)) * d
    sc.means3D[:] = (eye + d * fwd + lat * side + rng.normal(0, 0.05, (300, 3))).astype(np.float32)
    sc.scales[:] = np.exp(rng.uniform(-3, -1.5, (300, 3))).astype(np.float32)
    inp = mode_inputs(sc, ("shs", "sr"))
    cam = oracle_camera(view)
    ref = R.render(cam, inp["means3D"], inp["opacities"], shs=inp["shs"], scales=inp["scales"],
                   rotations=inp["rotations"])
    run = AbiRun(view, inp).forward()
    _check_integer_outputs(run, ref, cam)
    ok = ~ref.ambiguous
    assert np.abs(run.color.cpu().numpy() - ref.image)[:, ok].max() <= IMG_TOL
    dimg = rng.standard_normal((3, 96, 160)).astype(np.float32)
    gk, go = run.backward(dimg), ref.backward(dimg)
    for name, gref in go.items():
        assert rel_l2(gk[GRAD_NAMES[name]], gref) <= GRAD_TOL, name


def test_depth_ties_keep_gaussian_index_order():
    """Exact depth ties: the second half of the Gaussians repeats the first
    half's positions, scales and rotations (identical depth keys and tile
    rectangles) with their own opacities and colours.  Within a tile, tied
    Gaussians blend in index order (the stable sort of the reference's
    (tile, depth) keys), so the sorted values, the image and the gradients
    must match the oracle's order exactly."""
    sc = small_scene(P=1600, width=128, height=96, seed=13)
    half = sc.means3D.shape[0] // 2
    for a in (sc.means3D, sc.scales, sc.rotations):
        a[half:] = a[:half]
    view = sc.views[0]
    inp = mode_inputs(sc, ("shs", "sr"))
    cam = oracle_camera(view)
    ref = R.render(cam, inp["means3D"], inp["opacities"], shs=inp["shs"], scales=inp["scales"],
                   rotations=inp["rotations"])
    vis = ref.geom["visible"]
    assert vis[:half].any() and np.array_equal(vis[:half], vis[half:])
    run = AbiRun(view, inp).forward()
    dv = _check_integer_outputs(run, ref, cam)
    ok = ~ref.ambiguous
    assert np.abs(run.color.cpu().numpy() - ref.image)[:, ok].max() <= IMG_TOL
    np.testing.assert_array_equal(dv["n_contrib"][ok], ref.n_contrib[ok])
    dimg = np.random.default_rng(13).standard_normal((3, 96, 128)).astype(np.float32)
    gk, go = run.backward(dimg), ref.backward(dimg)
    for name, gref in go.items():
        assert rel_l2(gk[GRAD_NAMES[name]], gref) <= GRAD_TOL, name


def test_prefiltered_violation_is_an_error():
    sc = small_scene(P=100, width=32, height=32, seed=8)
    view = sc.views[0]
    inp = mode_inputs(sc, ("colors", "sr"))
    eye = view.campos.astype(np.float64)
    inp["means3D"][0] = (eye * 2.0).astype(np.float32)  # behind the camera
    from dmgs_gb300._lib import DmgsError
    with pytest.raises(DmgsError) as ei:
        AbiRun(view, inp, prefiltered=True).forward()
    assert ei.value.code == -4


def test_mark_visible_matches_oracle():
    from dmgs_gb300 import GaussianRasterizationSettings, GaussianRasterizer
    sc = small_scene(P=5000, seed=9)
    view = sc.views[0]
    d = "cuda"
    rs = GaussianRasterizationSettings(view.height, view.width, view.tanfovx, view.tanfovy,
                                       torch.zeros(3, device=d), 1.0,
                                       torch.tensor(view.viewmatrix, device=d),
                                       torch.tensor(view.projmatrix, device=d), 3,
                                       torch.tensor(view.campos, device=d), False, False)
    pts = np.random.default_rng(0).uniform(-8, 8, (5000, 3)).astype(np.float32)
    vis = GaussianRasterizer(rs).markVisible(torch.tensor(pts, device=d)).cpu().numpy()
    np.testing.assert_array_equal(vis, R.mark_visible(pts, view.viewmatrix))


def test_full_size_integer_outputs_bit_exact():
    """Configuration 3 at its full size (3M Gaussians of the large-scene
    generator, 1237x822): radii, tile rectangles, tiles touched, depth keys,
    the ~19M sorted (tile, depth) keys and Gaussian indices and the tile
    ranges all equal the oracle's float32 geometry and its stable sort; the
    ranges partition the instance list, and every listed Gaussian's rectangle
    contains its tile (size-independent properties of the same run)."""
    from dmgs_gb300.scenes import large_scene
    sc = large_scene(P=3_000_000, seed=0, n_views=1)
    view = sc.views[0]
    inp = mode_inputs(sc, ("shs", "sr"))
    run = AbiRun(view, inp, debug=False).forward()
    dv = run.debug_views()
    cam = oracle_camera(view)
    geom = R.geometry_f32(inp["means3D"], cam, inp["opacities"], inp["scales"], inp["rotations"])
    vis = geom["visible"]
    np.testing.assert_array_equal(run.radii.cpu().numpy()[:run.P], geom["radii"])
    np.testing.assert_array_equal(dv["rect"], np.where(vis[:, None], geom["rect"], 0))
    np.testing.assert_array_equal(dv["tiles_touched"], geom["tiles_touched"])
    np.testing.assert_array_equal(dv["depth"][vis].view(np.uint32), geom["depth"][vis].view(np.uint32))
    keys, vals, ranges = R.binning_fast(geom, cam)
    assert run.K == len(keys) > 10_000_000
    np.testing.assert_array_equal(dv["keys"], keys)
    np.testing.assert_array_equal(dv["values"], vals)
    np.testing.assert_array_equal(dv["ranges"], ranges)
    # properties: the non-empty ranges tile [0, K) in tile order; rectangles contain their tiles
    nz = ranges[:, 1] > ranges[:, 0]
    r = ranges[nz]
    assert r[0, 0] == 0 and r[-1, 1] == run.K and np.array_equal(r[1:, 0], r[:-1, 1])
    gx = (view.width + 15) // 16
    tiles = (dv["keys"] >> np.uint64(32)).astype(np.int64)
    rect = geom["rect"][dv["values"]]
    tx, ty = tiles % gx, tiles // gx
    assert np.all((rect[:, 0] <= tx) & (tx < rect[:, 2]) & (rect[:, 1] <= ty) & (ty < rect[:, 3]))


def _chain_magnitudes(inter, leaves, names):
    """Per Gaussian and input x, S(x) = sum over the nine 2D gradient
    components y_k (dL/dndc x, y; dL/dconic a, b, c; dL/dopacity; dL/drgb)
    of |d x / d y_k . dL/dy_k|: the first-order bound on the error of dL/dx
    when every 2D gradient carries a relative error of at most 1 (so e S(x)
    bounds it for a relative error e).  Computed on the oracle's FP64 graph."""
    import torch
    n = leaves[names[0]].shape[0]
    S = {k: torch.zeros(n, dtype=torch.float64) for k in names}
    comps = [("ndc", 0), ("ndc", 1), ("conic", 0), ("conic", 1), ("conic", 2), ("op", None),
             ("rgb", 0), ("rgb", 1), ("rgb", 2)]
    # the intermediates' gradients of the loss, taken before the calls below
    # (their retained-gradient hooks would add grad_outputs to them)
    dy = {k: inter[k].grad.clone() for k in ("ndc", "conic", "op", "rgb")}
    for name, c in comps:
        y = inter[name]
        go = torch.zeros_like(dy[name])
        if c is None:
            go.copy_(dy[name])
        else:
            go[:, c] = dy[name][:, c]
        gs = torch.autograd.grad(y, [leaves[k] for k in names], grad_outputs=go,
                                 retain_graph=True, allow_unused=True)
        for k, g in zip(names, gs):
            if g is not None:
                S[k] += g.reshape(n, -1).norm(dim=1)
    return {k: v.numpy() for k, v in S.items()}, {k: v.numpy() for k, v in dy.items()}


def test_full_size_sampled_tiles_image_and_gradients():
    """Configuration 3 at full size (3M Gaussians, 1237x822), 24 tiles spread
    over the view: the image matches the FP64 oracle blending of the same
    tile lists (pixels FP32 can decide); with dL/dimage non-zero only on those
    tiles:

    * the blend adjoint's per-Gaussian 2D gradients (NDC mean, conic,
      opacity, colour) match the oracle's intermediate gradients (1e-3
      relative L2);
    * the gradients of all five inputs match the oracle's autograd to 1e-3
      relative L2 over the Gaussians whose 3D gradient is well conditioned
      w.r.t. the 2D ones (the terms it sums cancel by less than 10x): all
      but a few tenths of a percent of them.  The rest are near-plane
      needles thousands of pixels long, whose position / shape gradient is
      the difference of chain terms up to 1000x larger than itself and whose
      blend exponent is the small difference of large float32 terms, so
      float32 arithmetic (the reference's too) cannot carry it to 1e-3; for
      them the error stays within 1e-2 of the magnitude of the terms summed;
    * the FP64-sum mode (dmgs_raster_bwd_f64sum) is run to run identical and
      meets the bars above; the default float-atomic adjoint meets them up
      to its own measured run-to-run spread (its summation order varies);
    * Gaussians that touch no sampled tile get zero.

    n_contrib (the position of the last blended Gaussian) may differ on a few
    pixels: after hundreds of factors the FP32 transmittance drifts by more
    than the oracle's 1e-5 relative ambiguity band around the 1e-4 stop, so
    the stop can move by one Gaussian whose contribution is below 1e-4 (the
    images still agree to 2e-4); the small-scene tests check it exactly."""
    import json
    import torch
    from dmgs_gb300.scenes import large_scene
    sc = large_scene(P=3_000_000, seed=0, n_views=1)
    view = sc.views[0]
    inp = mode_inputs(sc, ("shs", "sr"))
    run = AbiRun(view, inp, debug=False).forward()
    dv = run.debug_views()
    cam = oracle_camera(view)
    geom = R.geometry_f32(inp["means3D"], cam, inp["opacities"], inp["scales"], inp["rotations"])
    gx, gy = cam.grid
    tiles = np.linspace(0, gx * gy - 1, 24).astype(np.int64)
    vis = np.nonzero(geom["visible"])[0]
    rect = geom["rect"][vis]
    dbits = geom["depth"][vis].view(np.uint32)
    lists = []
    for t in tiles:
        ty, tx = divmod(int(t), gx)
        m = (rect[:, 0] <= tx) & (tx < rect[:, 2]) & (rect[:, 1] <= ty) & (ty < rect[:, 3])
        ids = vis[m]
        lists.append(ids[np.lexsort((ids, dbits[m]))])
    union = np.unique(np.concatenate(lists))
    assert len(union) > 1000
    f64 = lambda a: torch.tensor(np.asarray(a, np.float64), requires_grad=True)  # noqa: E731
    names = ("means3D", "opacities", "shs", "scales", "rotations")
    leaves = {k: f64(inp[k][union]) for k in names}
    ndc, pix, conic, op, rgb = R.project_fp64(cam, leaves["means3D"], leaves["opacities"],
                                              shs=leaves["shs"], scales=leaves["scales"],
                                              rotations=leaves["rotations"],
                                              sel=torch.arange(len(union)))
    inter = {"ndc": ndc, "conic": conic, "op": op, "rgb": rgb}
    for v in inter.values():
        v.retain_grad()
    pos = {int(g): i for i, g in enumerate(union)}
    rng = np.random.default_rng(3)
    dimg = np.zeros((3, view.height, view.width), np.float32)
    img = run.color.cpu().numpy()
    loss = 0.0
    checked = nc_diff = 0
    for t, ids in zip(tiles, lists):
        ty, tx = divmod(int(t), gx)
        x0, y0 = tx * 16, ty * 16
        x1, y1 = min(x0 + 16, view.width), min(y0 + 16, view.height)
        yy, xx = torch.meshgrid(torch.arange(y0, y1, dtype=torch.float64),
                                torch.arange(x0, x1, dtype=torch.float64), indexing="ij")
        pxy = torch.stack([xx.reshape(-1), yy.reshape(-1)], 1)
        g = torch.as_tensor([pos[int(i)] for i in ids], dtype=torch.long)
        out, _, nc, amb = R._blend_tile(pxy, pix[g], conic[g], op[g], rgb[g],
                                        torch.zeros(3, dtype=torch.float64))
        ok = ~amb.numpy()
        mine = img[:, y0:y1, x0:x1].reshape(3, -1).T
        assert np.abs(mine[ok] - out.detach().numpy()[ok]).max() <= IMG_TOL
        nc_diff += int((dv["n_contrib"][y0:y1, x0:x1].reshape(-1)[ok] != nc.numpy()[ok]).sum())
        d = rng.standard_normal(out.shape).astype(np.float32) * ok[:, None]
        dimg[:, y0:y1, x0:x1] = d.T.reshape(3, y1 - y0, x1 - x0)
        loss = loss + (out * torch.as_tensor(d, dtype=torch.float64)).sum()
        checked += int(ok.sum())
    assert checked > 5000
    assert nc_diff <= 0.02 * checked, (nc_diff, checked)
    loss.backward(retain_graph=True)
    S, dy = _chain_magnitudes(inter, leaves, names)

    g64 = run.backward(dimg, f64sum=True)
    rec = run.records2d[union].astype(np.float64)
    g64b = run.backward(dimg, f64sum=True)
    gfa = [run.backward(dimg) for _ in range(2)]  # float atomics
    rest = np.ones(run.P, bool)
    rest[union] = False
    # 2D records of the blend adjoint against the oracle's intermediate gradients
    e2d = {"ndc": rel_l2(rec[:, 0:2], dy["ndc"]), "conic": rel_l2(rec[:, 2:5], dy["conic"]),
           "opacity": rel_l2(rec[:, 5], dy["op"]), "rgb": rel_l2(rec[:, 6:9], dy["rgb"])}
    report = {"records_2d": e2d, "inputs": {}}
    for k in names:
        ref = leaves[k].grad.numpy().reshape(len(union), -1)
        mine = g64[GRAD_NAMES[k]][union].reshape(ref.shape).astype(np.float64)
        fa = [x[GRAD_NAMES[k]][union].reshape(ref.shape).astype(np.float64) for x in gfa]
        assert np.array_equal(g64[GRAD_NAMES[k]], g64b[GRAD_NAMES[k]]), k  # reproducible
        for x in (g64, *gfa):
            assert np.abs(x[GRAD_NAMES[k]][rest]).max() == 0.0, k
        gn = np.linalg.norm(ref, axis=1)
        cond = S[k] / np.maximum(gn, 1e-300)
        well = cond <= 10.0
        err = np.linalg.norm(mine - ref, axis=1)
        r = {"ill_conditioned": int((~well).sum()),
             "f64sum_vs_oracle_cond_le_100": rel_l2(mine[cond <= 100], ref[cond <= 100]),
             "f64sum_vs_oracle_cond_le_1000": rel_l2(mine[cond <= 1000], ref[cond <= 1000]),
             "cond_gt_100": int((cond > 100).sum()), "cond_max": float(cond.max()),
             "f64sum_vs_oracle_well": rel_l2(mine[well], ref[well]),
             "f64sum_vs_oracle_all": rel_l2(mine, ref),
             "atomics_vs_oracle_well": rel_l2(fa[0][well], ref[well]),
             "atomics_run_to_run_well": rel_l2(fa[1][well], fa[0][well]),
             "atomics_run_to_run_all": rel_l2(fa[1], fa[0]),
             "worst_err_over_S_ill": float((err[~well] / S[k][~well]).max()) if (~well).any() else 0.0}
        report["inputs"][k] = r
    print("FULL_SIZE_GRADIENTS", json.dumps(report))
    assert all(v <= GRAD_TOL for v in e2d.values()), e2d
    for k, r in report["inputs"].items():
        assert r["ill_conditioned"] <= 5e-3 * len(union), (k, r)
        assert r["f64sum_vs_oracle_well"] <= GRAD_TOL, (k, r)
        assert r["worst_err_over_S_ill"] <= 1e-2, (k, r)
        assert r["atomics_vs_oracle_well"] <= GRAD_TOL + 2 * r["atomics_run_to_run_well"], (k, r)
