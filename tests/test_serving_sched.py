"""Serving scheduler on the CPU with a fake device backend and a fake clock:
FIFO admission under the HBM budget and the slot limit, waves of at most
16 requests, overlap of waves in flight, and re-admission of a request whose
instance list overflowed with the exact count the device reported."""
import pytest

from dmgs_gb300.serving import CapacityEstimator, Request, Scheduler, poisson_trace


class View:
    def __init__(self, w, h):
        self.width, self.height = w, h


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def idle(self):
        self.t += 1e-4


class FakeBackend:
    """A wave completes `delay` seconds after launch; request r needs K(r)
    instances and overflows when its capacity is smaller."""

    def __init__(self, clock, delay=2e-3, bytes_per_pixel=10, K=lambda r: 1000 + 10 * r.scene):
        self.clock, self.delay, self.bpp, self.K = clock, delay, bytes_per_pixel, K
        self.launched, self.live_bytes, self.peak_live = [], 0, 0
        self.concurrent, self.peak_concurrent = 0, 0

    def footprint(self, r, cap):
        return self.bpp * r.view.width * r.view.height + 4 * cap

    def reserve(self, r, cap):
        return True

    def launch(self, reqs, caps, stream):
        nb = sum(self.footprint(r, c) for r, c in zip(reqs, caps))
        self.live_bytes += nb
        self.peak_live = max(self.peak_live, self.live_bytes)
        self.concurrent += 1
        self.peak_concurrent = max(self.peak_concurrent, self.concurrent)
        h = {"t": self.clock(), "reqs": list(reqs), "caps": list(caps), "bytes": nb, "stream": stream}
        self.launched.append(h)
        return h

    def ready(self, h):
        return self.clock() >= h["t"] + self.delay

    def results(self, h):
        out = []
        for r, c in zip(h["reqs"], h["caps"]):
            k = self.K(r)
            out.append((2 if k > c else 0, k))
            r.result = ("img", r.rid)
        return out

    def release(self, h):
        self.live_bytes -= h["bytes"]
        self.concurrent -= 1


def _reqs(n, t_step=1e-3, res=(64, 64), scenes=3):
    return [Request(i, i % scenes, View(*res), i * t_step) for i in range(n)]


def _sched(be, clk, **kw):
    est = kw.pop("estimator", CapacityEstimator(margin=1.0, slack=0, default=lambda r: 10**6))
    return Scheduler(be, clock=clk, idle=clk.idle, estimator=est, **kw)


def test_all_served_in_arrival_order_within_budget():
    clk = FakeClock()
    be = FakeBackend(clk)
    reqs = _reqs(200)
    budget = 5 * be.footprint(reqs[0], 10**6)
    st = _sched(be, clk, budget_bytes=budget).run(reqs)
    assert all(r.t_done >= r.arrival and r.result == ("img", r.rid) for r in reqs)
    admits = [r.t_admit for r in sorted(reqs, key=lambda r: r.arrival)]
    assert admits == sorted(admits)  # FIFO: never admitted ahead of an earlier arrival
    assert be.peak_live <= budget
    s = st.summary()
    assert s["requests"] == 200 and s["retries"] == 0 and s["p99_ms"] >= s["p50_ms"] > 0


def test_bursts_are_batched_into_waves_of_at_most_16_and_overlap():
    clk = FakeClock()
    be = FakeBackend(clk, delay=5e-3)
    reqs = [Request(i, i % 4, View(32, 32), 0.0) for i in range(40)]  # one burst
    st = _sched(be, clk, budget_bytes=10**12, max_inflight=64, n_streams=4).run(reqs)
    sizes = [len(h["reqs"]) for h in be.launched]
    assert sizes == [16, 16, 8] and st.waves == 3
    assert be.peak_concurrent == 3  # all three waves in flight at once
    assert {h["stream"] for h in be.launched} == {0, 1, 2}


def test_slot_limit_bounds_requests_in_flight():
    clk = FakeClock()
    be = FakeBackend(clk, delay=5e-3)
    reqs = [Request(i, 0, View(32, 32), 0.0) for i in range(30)]
    st = _sched(be, clk, budget_bytes=10**12, max_inflight=8).run(reqs)
    assert st.peak_inflight == 8 and all(len(h["reqs"]) <= 8 for h in be.launched)


def test_overflow_is_retried_with_the_reported_count():
    clk = FakeClock()
    be = FakeBackend(clk, K=lambda r: 5000)
    est = CapacityEstimator(margin=1.0, slack=0, default=lambda r: 100)  # too small at first
    reqs = _reqs(10, t_step=1e-2, scenes=1)
    st = _sched(be, clk, budget_bytes=10**9, estimator=est).run(reqs)
    assert st.retries == 1  # the first request; later ones use the observed count
    assert reqs[0].attempts == 2 and all(r.attempts == 1 for r in reqs[1:])
    assert [c for h in be.launched for c in h["caps"]][:2] == [100, 5000]
    assert all(r.result is not None for r in reqs)


def test_request_above_the_budget_is_refused():
    clk = FakeClock()
    be = FakeBackend(clk)
    with pytest.raises(RuntimeError, match="above the budget"):
        _sched(be, clk, budget_bytes=100).run(_reqs(2))


def test_poisson_trace_rate_and_mix():
    reqs = poisson_trace(200.0, 5.0, 8, [(256, 256), (800, 800)], seed=3,
                         view_fn=lambda rng, w, h: View(w, h))
    assert 850 < len(reqs) < 1150
    assert sorted(r.arrival for r in reqs) == [r.arrival for r in reqs]
    assert {r.scene for r in reqs} == set(range(8))
    assert {(r.view.width, r.view.height) for r in reqs} == {(256, 256), (800, 800)}


def test_device_arena_first_fit_and_coalescing():
    torch = pytest.importorskip("torch")
    from dmgs_gb300.serving import DeviceArena
    a = DeviceArena(4096, torch.device("cpu"))
    x = a.alloc(1000)   # 1024
    y = a.alloc(100)    # 256
    z = a.alloc(2000)   # 2048
    assert (x, y, z) == (0, 1024, 1280) and a.alloc(1024) is None  # 768 left
    a.release(y, 100)
    assert a.alloc(300) == 3328 and a.alloc(200) == 1024  # first fit: tail, then the hole
    assert a.alloc(256) == 3840 and a.alloc(1) is None
    for o, n in [(1024, 200), (3328, 300), (3840, 256)]:
        a.release(o, n)
    a.release(x, 1000)
    a.release(z, 2000)
    assert a.free == [(0, 4096)] and a.used == 0
    t = a.tensor(256, 6, torch.float32, (2, 3))
    assert t.shape == (2, 3) and t.data_ptr() == a.base + 256


def test_admission_timeout_drops_requests_never_admitted():
    """One wave at a time (the budget fits one request), 10 ms per wave: of a
    burst of 6 requests allowed 25 ms to be admitted, the first three are
    served and the rest time out unrendered."""
    clk = FakeClock()
    be = FakeBackend(clk, delay=10e-3)
    reqs = [Request(i, 0, View(32, 32), 0.0, admit_timeout=25e-3) for i in range(6)]
    delivered = []
    est = CapacityEstimator(margin=1.0, slack=0, default=lambda r: 1000)
    st = _sched(be, clk, budget_bytes=be.footprint(reqs[0], 1000),
                estimator=est).run(reqs, deliver=delivered.append)
    launched = [r.rid for h in be.launched for r in h["reqs"]]
    assert launched == [0, 1, 2]
    assert [r.status for r in reqs] == ["done"] * 3 + ["timeout"] * 3
    assert [r.rid for r in delivered] == [0, 1, 2]
    assert all(r.result is None for r in reqs[3:])
    s = st.summary()
    assert s["requests"] == 3 and s["timeouts"] == 3 and s["cancelled"] == 0


def test_timeout_does_not_drop_an_overflow_retry():
    clk = FakeClock()
    be = FakeBackend(clk, delay=10e-3, K=lambda r: 5000)
    est = CapacityEstimator(margin=1.0, slack=0, default=lambda r: 100)  # overflows first
    reqs = [Request(0, 0, View(32, 32), 0.0, admit_timeout=1e-3)]
    st = _sched(be, clk, budget_bytes=10**9, estimator=est).run(reqs)
    assert reqs[0].status == "done" and reqs[0].attempts == 2 and st.timeouts == 0


def test_cancellation_before_admission_and_while_rendering():
    """Arrivals every 1 ms, 4 ms per wave.  Request 3 is cancelled before it
    arrives; when request 0 is delivered (t = 4 ms) the client cancels
    request 2 (its wave is running: rendered, result dropped), request 1
    (running and about to overflow: not retried) and request 6 (not yet
    arrived: never rendered)."""
    clk = FakeClock()
    be = FakeBackend(clk, delay=4e-3, K=lambda r: 5000 if r.rid == 1 else 1000)
    est = CapacityEstimator(margin=1.0, slack=0, default=lambda r: 2000)
    reqs = [Request(i, 0, View(32, 32), 1e-3 * i) for i in range(10)]
    reqs[3].cancelled = True
    sched = _sched(be, clk, budget_bytes=10**9, estimator=est)
    delivered = []

    def deliver(r):
        delivered.append(r.rid)
        if r.rid == 0:
            for k in (2, 1, 6):
                sched.cancel(reqs[k])

    st = sched.run(reqs, deliver=deliver)
    launched = sorted(r.rid for h in be.launched for r in h["reqs"])
    assert launched == [0, 1, 2, 4, 5, 7, 8, 9]
    status = {r.rid: r.status for r in reqs}
    assert [k for k, v in status.items() if v == "cancelled"] == [1, 2, 3, 6]
    assert all(status[k] == "done" for k in (0, 4, 5, 7, 8, 9))
    assert delivered == [0, 4, 5, 7, 8, 9]
    assert all(reqs[k].result is None for k in (1, 2, 3, 6))
    assert st.cancelled == 4 and st.retries == 0 and st.summary()["requests"] == 6
