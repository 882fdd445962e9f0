"""The multi-view batched form against the per-view drop-in path and the
oracle: images must be bit-identical to the per-view path for every blend
configuration (same per-pixel arithmetic and order), summed gradients equal
the per-view sum, capacity overflow is reported without faulting, and CUDA
graph replays reproduce eager results and follow in-place parameter updates."""
import numpy as np
import pytest
import torch

import dmgs_gb300
from dmgs_gb300._lib import DmgsError
from dmgs_gb300.batched import TUNE_SPACE, BatchedRasterizer, autotune, rasterize_batched
from dmgs_gb300.scenes import random_inside_view, small_scene
from helpers import oracle_camera, rel_l2
from oracle import raster as R

pytestmark = pytest.mark.gpu
D = "cuda"


def _settings(view, deg=3, bg=(0.0, 0.0, 0.0)):
    return dmgs_gb300.GaussianRasterizationSettings(
        image_height=view.height, image_width=view.width, tanfovx=view.tanfovx,
        tanfovy=view.tanfovy, bg=torch.tensor(bg, dtype=torch.float32, device=D),
        scale_modifier=1.0, viewmatrix=torch.tensor(view.viewmatrix, device=D),
        projmatrix=torch.tensor(view.projmatrix, device=D), sh_degree=deg,
        campos=torch.tensor(view.campos, device=D), prefiltered=False, debug=False)


def _scene_and_views(P=6000, seed=41):
    sc = small_scene(P=P, seed=seed)
    rng = np.random.default_rng(seed)
    res = [(96, 80), (160, 128), (64, 64), (200, 120)]
    views = []
    for i in range(5):
        w, h = res[i % len(res)]
        a = rng.uniform(0, 2 * np.pi)
        eye = 3.5 * np.array([np.cos(a), rng.uniform(-0.5, 0.8), np.sin(a)])
        from dmgs_gb300.camera import make_view
        views.append(make_view(eye, (0, 0, 0), w, h, fovx_deg=50))
    return sc, views


def _gauss(sc):
    return {"means3D": torch.tensor(sc.means3D, device=D), "opacities": torch.tensor(sc.opacities, device=D),
            "shs": torch.tensor(sc.shs, device=D), "scales": torch.tensor(sc.scales, device=D),
            "rotations": torch.tensor(sc.rotations, device=D)}


def _plain(g, rs, dimg):
    t = {k: v.clone().requires_grad_(True) for k, v in g.items()}
    m2 = torch.zeros_like(t["means3D"], requires_grad=True)
    img, radii = dmgs_gb300.GaussianRasterizer(rs)(means3D=t["means3D"], means2D=m2,
                                                    opacities=t["opacities"], shs=t["shs"],
                                                    scales=t["scales"], rotations=t["rotations"])
    img.backward(dimg)
    return img.detach(), {k: v.grad for k, v in t.items()}, m2.grad


def test_batched_matches_per_view_path_for_every_config():
    sc, views = _scene_and_views()
    g = _gauss(sc)
    settings = [_settings(v) for v in views]
    gen = torch.Generator(device=D).manual_seed(3)
    dimgs = [torch.randn(3, v.height, v.width, device=D, generator=gen) for v in views]
    plain = [_plain(g, rs, d) for rs, d in zip(settings, dimgs)]
    gsum = {k: sum(p[1][k] for p in plain) for k in g}
    br = BatchedRasterizer(settings, g)
    for ppt, b, shape in TUNE_SPACE:
        br.set_config(ppt, b, shape)
        br.forward()
        br.backward(dimgs)
        torch.cuda.synchronize()
        br.status()
        for v in range(len(views)):
            assert torch.equal(br.images[v], plain[v][0]), (ppt, b, shape, v)
            assert torch.equal(br.radii[v], dmgs_gb300.GaussianRasterizer(settings[v])(
                means3D=g["means3D"], means2D=torch.zeros_like(g["means3D"]), opacities=g["opacities"],
                shs=g["shs"], scales=g["scales"], rotations=g["rotations"])[1])
            assert rel_l2(br.means2D_grads[v].cpu().numpy(), plain[v][2].cpu().numpy()) <= 1e-5
        for k in g:
            assert rel_l2(br.grads[k].cpu().numpy(), gsum[k].cpu().numpy()) <= 1e-5, (ppt, b, shape, k)


def test_batched_against_oracle():
    sc, views = _scene_and_views(P=2500, seed=42)
    views = views[:3]
    g = _gauss(sc)
    br = BatchedRasterizer([_settings(v) for v in views], g)
    rng = np.random.default_rng(4)
    dimgs = [rng.standard_normal((3, v.height, v.width)).astype(np.float32) for v in views]
    br.forward()
    br.backward([torch.tensor(d, device=D) for d in dimgs])
    torch.cuda.synchronize()
    gsum = None
    for v, view in enumerate(views):
        ref = R.render(oracle_camera(view), sc.means3D, sc.opacities, shs=sc.shs, scales=sc.scales,
                       rotations=sc.rotations)
        ok = ~ref.ambiguous
        assert np.abs(br.images[v].cpu().numpy() - ref.image)[:, ok].max() <= 2e-4
        gv = ref.backward(dimgs[v])
        gsum = gv if gsum is None else {k: gsum[k] + gv[k] for k in gsum}
    for k in ("means3D", "opacities", "shs", "scales", "rotations"):
        assert rel_l2(br.grads[k].cpu().numpy(), gsum[k]) <= 1e-3, k


def test_capacity_overflow_is_reported_not_faulted():
    sc, views = _scene_and_views(P=3000, seed=43)
    g = _gauss(sc)
    br = BatchedRasterizer([_settings(v, bg=(0.25, 0.5, 0.75)) for v in views[:2]], g,
                           capacity=[10, 10**7])
    br.forward()
    br.backward([torch.ones_like(i) for i in br.images])
    torch.cuda.synchronize()
    with pytest.raises(DmgsError) as ei:
        br.status()
    assert ei.value.code == -5
    # the overflowing view rendered background only; the other view is intact
    bg = torch.tensor([0.25, 0.5, 0.75], device=D).view(3, 1, 1).expand_as(br.images[0])
    assert torch.equal(br.images[0], bg)
    assert not torch.equal(br.images[1], torch.zeros_like(br.images[1]))
    br.grow()
    br.forward()
    torch.cuda.synchronize()
    br.status()


def test_graph_replay_matches_eager_and_follows_parameter_updates():
    sc, views = _scene_and_views(P=4000, seed=44)
    g = _gauss(sc)
    settings = [_settings(v) for v in views[:4]]
    br = BatchedRasterizer(settings, g)
    gen = torch.Generator(device=D).manual_seed(5)
    for d in br.dL_dout:
        d.copy_(torch.randn(d.shape, device=D, generator=gen))
    br.step()
    torch.cuda.synchronize()
    eager_imgs = [i.clone() for i in br.images]
    eager_grads = {k: v.clone() for k, v in br.grads.items() if v is not None}
    br.capture()
    br.step()
    torch.cuda.synchronize()
    for a, b in zip(eager_imgs, br.images):
        assert torch.equal(a, b)
    for k, v in eager_grads.items():
        assert rel_l2(br.grads[k].cpu().numpy(), v.cpu().numpy()) <= 1e-5, k
    # an in-place parameter update is seen by the next replay
    with torch.no_grad():
        br.g["means3D"].add_(0.01)
    br.step()
    torch.cuda.synchronize()
    br.status()
    moved = dmgs_gb300.GaussianRasterizer(settings[0])(
        means3D=br.g["means3D"], means2D=torch.zeros_like(br.g["means3D"]), opacities=g["opacities"],
        shs=g["shs"], scales=g["scales"], rotations=g["rotations"])[0]
    assert torch.equal(br.images[0], moved)


def test_autotune_and_autograd_entry(tmp_path):
    sc, views = _scene_and_views(P=3000, seed=45)
    g = _gauss(sc)
    br = BatchedRasterizer([_settings(v) for v in views[:3]], g)
    res = autotune(br, iters=2, cache_path=str(tmp_path / "tune.json"))
    assert tuple(res["best"]) in TUNE_SPACE and len(res["ms"]) == len(TUNE_SPACE)
    again = autotune(br, cache_path=str(tmp_path / "tune.json"))
    assert again["best"] == res["best"]
    leaves = {k: v.clone().requires_grad_(True) for k, v in g.items()}
    br2 = BatchedRasterizer([_settings(v) for v in views[:3]], leaves)
    imgs = rasterize_batched(br2, leaves["means3D"], leaves["opacities"], shs=leaves["shs"],
                             scales=leaves["scales"], rotations=leaves["rotations"])
    sum(i.sum() for i in imgs).backward()
    ref = [_plain(g, _settings(v), torch.ones(3, v.height, v.width, device=D)) for v in views[:3]]
    for k in g:
        assert rel_l2(leaves[k].grad.cpu().numpy(), sum(r[1][k] for r in ref).cpu().numpy()) <= 1e-5, k


def test_fused_densification_stats_match_per_view_gradients():
    sc, views = _scene_and_views(P=4000, seed=46)
    g = _gauss(sc)
    settings = [_settings(v) for v in views]
    br = BatchedRasterizer(settings, g, means2D_grads=True, densify_stats=True)
    gen = torch.Generator(device=D).manual_seed(6)
    dimgs = [torch.randn(3, v.height, v.width, device=D, generator=gen) for v in views]
    br.forward()
    br.backward(dimgs)
    torch.cuda.synchronize()
    acc = torch.zeros(br.P, device=D)
    cnt = torch.zeros(br.P, device=D)
    for v in range(len(views)):
        vis = br.radii[v] > 0
        acc[vis] += br.means2D_grads[v][vis, :2].norm(dim=-1)
        cnt[vis] += 1
        assert torch.all(br.means2D_grads[v][~vis] == 0)  # zero where not visible
    assert torch.equal(br.densify_count, cnt)
    assert torch.allclose(br.densify_accum, acc, rtol=1e-5, atol=1e-12)
    br.forward()
    br.backward()  # same gradients again: the statistics accumulate
    torch.cuda.synchronize()
    assert torch.equal(br.densify_count, 2 * cnt)
    assert torch.allclose(br.densify_accum, 2 * acc, rtol=1e-5, atol=1e-12)
    br.reset_densify_stats()
    assert not br.densify_accum.any() and not br.densify_count.any()
    # without per-view outputs the summed parameter gradients are unchanged
    lean = BatchedRasterizer(settings, g, means2D_grads=False)
    lean.forward()
    lean.backward(dimgs)
    torch.cuda.synchronize()
    for k in g:
        assert rel_l2(lean.grads[k].cpu().numpy(), br.grads[k].cpu().numpy()) <= 1e-5, k


def test_host_pipeline_overlapped_steps_match_the_direct_step():
    from dmgs_gb300.batched import HostPipeline
    sc, views = _scene_and_views(P=3000, seed=47)
    g = _gauss(sc)
    settings = [_settings(v) for v in views[:3]]
    gen = torch.Generator(device=D).manual_seed(8)
    names = list(g)
    pipe = HostPipeline(settings, g, names)
    steps = []
    for i in range(4):  # different parameters and image gradients every step
        params = {k: (v + 0.001 * i).cpu().pin_memory() for k, v in g.items()}
        douts = [torch.randn(3, v.height, v.width, device=D, generator=gen).cpu().pin_memory()
                 for v in views[:3]]
        imgs = [torch.empty(3, v.height, v.width).pin_memory() for v in views[:3]]
        grads = {k: torch.empty(g[k].shape).pin_memory() for k in names}
        steps.append((params, douts, imgs, grads))
    pipe.start()
    for st in steps:
        pipe.submit(*st)
    pipe.finish()
    torch.cuda.synchronize()
    for params, douts, imgs, grads in steps:
        br = BatchedRasterizer(settings, {k: v.to(D) for k, v in params.items()})
        br.forward()
        br.backward([d.to(D) for d in douts])
        torch.cuda.synchronize()
        for a, b in zip(imgs, br.images):
            assert torch.equal(a, b.cpu())
        for k in names:
            assert rel_l2(grads[k].numpy(), br.grads[k].cpu().numpy()) <= 1e-5, k


def test_view_with_nothing_visible_in_a_batch():
    from dmgs_gb300.camera import make_view
    sc, views = _scene_and_views(P=2000, seed=48)
    g = _gauss(sc)
    away = make_view((0.0, 0.0, 3.5), (0.0, 0.0, 10.0), 90, 70, fovx_deg=40)  # facing away
    settings = [_settings(away, bg=(0.2, 0.3, 0.4)), _settings(views[0])]
    br = BatchedRasterizer(settings, g)
    assert br.count_instances()[0] == 0
    br.forward()
    br.backward([torch.ones_like(i) for i in br.images])
    torch.cuda.synchronize()
    br.status()
    bg = torch.tensor([0.2, 0.3, 0.4], device=D).view(3, 1, 1).expand_as(br.images[0])
    assert torch.equal(br.images[0], bg)
    assert torch.count_nonzero(br.radii[0]) == 0
    plain = _plain(g, settings[1], torch.ones(3, views[0].height, views[0].width, device=D))
    assert torch.equal(br.images[1], plain[0])
    for k in g:  # the empty view adds nothing to the summed gradients
        assert rel_l2(br.grads[k].cpu().numpy(), plain[1][k].cpu().numpy()) <= 1e-5, k


def test_inside_views_with_mixed_modifiers_and_given_covariances_match_per_view_path():
    """Cameras inside a large-scene cloud, where most (Gaussian, view) pairs
    lie behind the camera or off screen and the batched preprocess culls them
    by its conservative pre-test: radii and images bit-identical to the
    per-view path, with views of other scale modifiers in the batch (no
    pre-test bound for them when the covariance comes from scale and
    rotation) and with given 3D covariances."""
    from dmgs_gb300.scenes import large_scene
    sc = large_scene(P=200_000, seed=7, n_views=1)
    rng = np.random.default_rng(77)
    views = [random_inside_view(rng, 320, 240) for _ in range(6)]
    mods = [1.0, 1.0, 0.6, 1.0, 1.7, 1.0]
    base = _gauss(sc)
    cov = R.cov3d_from_scale_rot_f32(sc.scales, sc.rotations, np.float32(1.0))
    given = {"means3D": base["means3D"], "opacities": base["opacities"], "shs": base["shs"],
             "cov3D_precomp": torch.tensor(np.ascontiguousarray(cov, np.float32), device=D)}
    for g in (base, given):
        settings = [_settings(v)._replace(scale_modifier=m) for v, m in zip(views, mods)]
        br = BatchedRasterizer(settings, g, means2D_grads=False)
        br.forward()
        torch.cuda.synchronize()
        br.status()
        for v, rs in enumerate(settings):
            img, radii = dmgs_gb300.GaussianRasterizer(rs)(means2D=torch.zeros_like(g["means3D"]), **g)
            assert torch.count_nonzero(radii) > 1000, v
            assert torch.equal(br.radii[v], radii), (sorted(g), v)
            assert torch.equal(br.images[v], img), (sorted(g), v)
            # the per-view path runs the same pre-test: pin both on the FP32 oracle
            cam = oracle_camera(views[v], scale_modifier=mods[v])
            if "cov3D_precomp" in g:
                geom = R.geometry_f32(sc.means3D, cam, sc.opacities, cov3D=cov)
            else:
                geom = R.geometry_f32(sc.means3D, cam, sc.opacities, sc.scales, sc.rotations)
            np.testing.assert_array_equal(br.radii[v].cpu().numpy(), geom["radii"])


def test_configuration4_full_size_graph_matches_plain_and_oracle():
    """Configuration 4 at its full size: the 3M-Gaussian large scene, 16
    views at 400x400, 800x800, 1237x822 and 1600x900 round-robin, forward +
    backward replayed from the captured CUDA graph.  Every view's image and
    radii are bit-identical to the plain drop-in's (one view per call), each
    view's screen-space gradient and the gradients summed over the views
    match the per-view sums up to the float atomics' summation order (bounded
    by the spread between two replays of the batched step itself, plus 1e-5);
    the 1600x900 view's image matches the FP64 oracle on 24 sampled tiles."""
    from dmgs_gb300.scenes import large_scene
    from helpers import blend_sampled_tiles, sampled_tile_lists
    sc = large_scene(P=3_000_000, seed=0, n_views=1)
    g = _gauss(sc)
    rng = np.random.default_rng(1234)
    mixed = [(400, 400), (800, 800), (1237, 822), (1600, 900)]
    views = [random_inside_view(rng, *mixed[i % 4]) for i in range(16)]
    settings = [_settings(v) for v in views]
    gen = torch.Generator(device=D).manual_seed(5)
    dimgs = [torch.randn(3, v.height, v.width, device=D, generator=gen) for v in views]
    br = BatchedRasterizer(settings, g, means2D_grads=True)
    for dst, src in zip(br.dL_dout, dimgs):
        dst.copy_(src)
    br.capture()
    br.step()
    torch.cuda.synchronize()
    br.status()
    grads1 = {k: v.clone() for k, v in br.grads.items() if v is not None}
    m2_1 = [m.clone() for m in br.means2D_grads]
    images = [i.clone() for i in br.images]
    radii = [r.clone() for r in br.radii]
    br.step()  # a second replay: the run-to-run spread of the float atomics
    torch.cuda.synchronize()
    gsum = {k: torch.zeros_like(v) for k, v in grads1.items()}
    for v in range(16):
        img, gv, m2 = _plain(g, settings[v], dimgs[v])
        assert torch.equal(images[v], img), v
        rp = dmgs_gb300.GaussianRasterizer(settings[v])(
            means3D=g["means3D"], means2D=torch.zeros_like(g["means3D"]), opacities=g["opacities"],
            shs=g["shs"], scales=g["scales"], rotations=g["rotations"])[1]
        assert torch.equal(radii[v], rp), v
        spread = rel_l2(br.means2D_grads[v].cpu().numpy(), m2_1[v].cpu().numpy())
        assert rel_l2(m2_1[v].cpu().numpy(), m2.cpu().numpy()) <= 1e-5 + 4 * spread, v
        for k in gsum:
            gsum[k] += gv[k]
    for k in gsum:
        spread = rel_l2(br.grads[k].cpu().numpy(), grads1[k].cpu().numpy())
        e = rel_l2(grads1[k].cpu().numpy(), gsum[k].cpu().numpy())
        assert e <= 1e-5 + 4 * spread, (k, e, spread)
    # the 1600x900 view against the FP64 oracle on sampled tiles
    vi = 3
    view = views[vi]
    cam = oracle_camera(view)
    geom = R.geometry_f32(sc.means3D, cam, sc.opacities, sc.scales, sc.rotations)
    gx, gy = cam.grid
    tiles = np.linspace(0, gx * gy - 1, 24).astype(np.int64)
    lists, union = sampled_tile_lists(geom, gx, tiles)
    assert len(union) > 1000
    f64 = lambda a: torch.tensor(np.asarray(a, np.float64))  # noqa: E731
    _, pix, conic, op, rgb = R.project_fp64(cam, f64(sc.means3D[union]), f64(sc.opacities[union]),
                                            shs=f64(sc.shs[union]), scales=f64(sc.scales[union]),
                                            rotations=f64(sc.rotations[union]),
                                            sel=torch.arange(len(union)))
    _, _, err, checked = blend_sampled_tiles(view.width, view.height, gx, tiles, lists, union, pix,
                                             conic, op, rgb, (0.0, 0.0, 0.0),
                                             images[vi].cpu().numpy())
    assert checked > 5000 and err <= 2e-4, (checked, err)
