"""Serving loop on the GPU: every request's image is bit-identical whether
it is rendered alone, in a mixed wave with requests for other scenes and
resolutions, after a capacity-overflow retry, or by the plain drop-in
rasteriser; a short Poisson trace is served in real time."""
import numpy as np
import pytest
import torch

import dmgs_gb300
from dmgs_gb300.scenes import large_scene_tensors, random_inside_view
from dmgs_gb300.serving import (CapacityEstimator, GpuBackend, Request, ResidentScene, Scheduler,
                                poisson_trace, profile_capacity)

pytestmark = pytest.mark.gpu
D = torch.device("cuda")
RES = [(96, 80), (160, 128), (256, 256), (200, 120)]


@pytest.fixture(scope="module")
def scenes():
    return [ResidentScene(large_scene_tensors(P, seed, D)) for P, seed in
            [(30000, 1), (60000, 2), (15000, 3)]]


def _views(n, seed=0):
    rng = np.random.default_rng(seed)
    return [(i % 3, random_inside_view(rng, *RES[i % len(RES)])) for i in range(n)]


def _plain(scene, v):
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=D)  # noqa: E731
    rs = dmgs_gb300.GaussianRasterizationSettings(
        image_height=v.height, image_width=v.width, tanfovx=v.tanfovx, tanfovy=v.tanfovy,
        bg=torch.zeros(3, device=D), scale_modifier=1.0, viewmatrix=t(v.viewmatrix),
        projmatrix=t(v.projmatrix), sh_degree=3, campos=t(v.campos), prefiltered=False, debug=False)
    with torch.no_grad():
        img, _ = dmgs_gb300.GaussianRasterizer(rs)(
            means3D=scene.t["means3D"], means2D=None, opacities=scene.t["opacities"],
            shs=scene.t["shs"], scales=scene.t["scales"], rotations=scene.t["rotations"])
    return img.cpu()


def _serve(scenes, views, est, **kw):
    reqs = [Request(i, s, v, 0.0) for i, (s, v) in enumerate(views)]
    st = Scheduler(GpuBackend(scenes, 1 << 31, n_streams=3), 1 << 31, estimator=est, **kw).run(reqs)
    return reqs, st


def test_results_identical_alone_in_the_mix_and_plain(scenes):
    views = _views(12)
    est = profile_capacity(scenes, RES, n_views=2)
    alone, st1 = _serve(scenes, views, est, max_wave=1, max_inflight=1)
    mix, st2 = _serve(scenes, views, est, max_wave=16)
    assert st1.waves == 12 and st2.waves == 1  # one burst: a single wave of all 12
    for (s, v), a, m in zip(views, alone, mix):
        assert torch.equal(a.result, m.result)
        assert torch.equal(m.result, _plain(scenes[s], v))
        assert m.result.abs().sum() > 0


def test_overflow_retry_gives_the_same_images(scenes):
    views = _views(6, seed=1)
    tiny = CapacityEstimator(margin=1.0, slack=0, default=lambda r: 64)
    reqs, st = _serve(scenes, views, tiny, max_wave=16)
    assert st.retries == 6 and all(r.attempts == 2 for r in reqs)  # each first attempt overflows
    for (s, v), r in zip(views, reqs):
        assert torch.equal(r.result, _plain(scenes[s], v))


def test_poisson_trace_in_real_time(scenes):
    reqs = poisson_trace(400.0, 0.25, len(scenes), RES, seed=2)
    est = profile_capacity(scenes, RES, n_views=2)
    be = GpuBackend(scenes, 1 << 31, n_streams=4)
    st = Scheduler(be, 1 << 31, estimator=est).run(reqs, deliver=be.recycle)
    s = st.summary()
    assert s["requests"] == len(reqs) > 50
    assert 0 < s["p50_ms"] <= s["p99_ms"] < 1000


def test_empty_and_culled_scenes_render_background(scenes):
    from dmgs_gb300.camera import make_view
    empty = ResidentScene({k: v[:0] for k, v in scenes[0].t.items()})
    mixed = [scenes[0], empty]
    away = make_view((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 64, 48, fovx_deg=1.0)  # a sliver of sky
    views = [(1, random_inside_view(np.random.default_rng(3), 96, 80)), (0, away), (0, _views(1)[0][1])]
    est = CapacityEstimator(margin=1.0, slack=1024, default=lambda r: 1 << 16)
    reqs = [Request(i, s, v, 0.0) for i, (s, v) in enumerate(views)]
    Scheduler(GpuBackend(mixed, 1 << 30, n_streams=2), 1 << 30, estimator=est).run(reqs)
    assert torch.count_nonzero(reqs[0].result) == 0  # empty scene: black background
    for (s, v), r in zip(views[1:], reqs[1:]):
        assert torch.equal(r.result, _plain(mixed[s], v))
