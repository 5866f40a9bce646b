"""Serving loop scheduling on the host: admission by a device-memory budget,
cohorts, one frame per tick, retirement and memory release.  A fake solver
back end stands in for the GPU (no device is touched)."""
import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.serving import ClothRequest, ServingEngine, estimate_device_bytes


class FakeSolver:
    def __init__(self, reqs):
        self.reqs = reqs
        self.frames = 0
        self.active = [True] * len(reqs)
        self.closed = False

    def positions(self, k):
        n = len(self.reqs[k].cloth.positions_world)
        return np.full((n, 3), float(self.reqs[k].request_id), np.float32)


class FakeBackend:
    def __init__(self):
        self.created = []
        self.steps = 0

    def create(self, reqs):
        s = FakeSolver(reqs)
        self.created.append(s)
        return s

    @staticmethod
    def device_bytes(solver):
        return sum(estimate_device_bytes(r) for r in solver.reqs)

    def step(self, solver, substeps, iterations):
        assert not solver.closed
        solver.frames += 1
        self.steps += 1

    @staticmethod
    def wait(solver):
        pass

    @staticmethod
    def download(solver, slot, batched):
        assert solver.active[slot]
        return solver.positions(slot)

    @staticmethod
    def deactivate(solver, slot, batched):
        solver.active[slot] = False

    @staticmethod
    def close(solver):
        solver.closed = True


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 0.001
        return self.t


def _req(rid, side, frames, arrival=0.0):
    cloth = scene._unpinned_grid(side, 0.5)
    opt = scene.SolverOptions(self_collision=True, self_collision_mode=2, cloth_thickness=0.002, collision_margin=0.002)
    return ClothRequest(cloth, opt, np.empty((0, 3, 3), np.float32), frames, 10, 2, rid, arrival)


def test_budget_fifo_and_release():
    reqs = [_req(k, 40, 3 + k) for k in range(6)]
    one = estimate_device_bytes(reqs[0])
    be = FakeBackend()
    eng = ServingEngine(hbm_budget_bytes=int(2.5 * one), backend=be, clock=FakeClock(), workers=0)
    for r in reqs:
        eng.submit(r)
    done, order, ticks = [], [], 0
    while not eng.idle():
        assert eng.used_bytes <= eng.budget
        for res in eng.tick():
            done.append(res)
            order.append(res.request_id)
        ticks += 1
        assert ticks < 100
    assert sorted(order) == list(range(6))
    for res in done:
        assert res.frames == 3 + res.request_id
        assert np.all(res.positions == res.request_id)
    assert eng.used_bytes == 0 and eng.peak_bytes <= eng.budget
    assert all(s.closed for s in be.created)
    # two fit at once: the third waits until memory is released
    assert len(be.created[0].reqs) == 2


def test_small_requests_share_cohorts_large_alone():
    be = FakeBackend()
    eng = ServingEngine(hbm_budget_bytes=1 << 40, group_below=5000, backend=be, clock=FakeClock(), workers=0)
    for k, side in enumerate([20, 30, 25, 90, 100]):  # 400, 900, 625 grouped; 8100, 10000 alone
        eng.submit(_req(k, side, 4))
    eng.tick()
    sizes = sorted(len(s.reqs) for s in be.created)
    assert sizes == [1, 1, 3]
    while not eng.idle():
        eng.tick()
    assert be.steps == 3 * 4  # three cohorts, four frames each


def test_requests_join_between_ticks():
    be = FakeBackend()
    eng = ServingEngine(hbm_budget_bytes=1 << 40, backend=be, clock=FakeClock(), workers=0)
    eng.submit(_req(0, 20, 5))
    eng.tick()
    eng.tick()
    eng.submit(_req(1, 20, 2))  # arrives while request 0 is resident
    finished = []
    while not eng.idle():
        finished += [r.request_id for r in eng.tick()]
    assert finished == [1, 0]  # 1 runs ticks 3-4, 0 runs ticks 1-5
    assert len(be.created) == 2


def test_request_over_whole_budget_is_refused():
    eng = ServingEngine(hbm_budget_bytes=1000, backend=FakeBackend(), clock=FakeClock(), workers=0)
    eng.submit(_req(0, 20, 1))
    with pytest.raises(MemoryError):
        eng.tick()


def test_run_with_arrivals_reports_latency():
    be = FakeBackend()
    eng = ServingEngine(hbm_budget_bytes=1 << 40, backend=be, clock=FakeClock(), workers=0)
    reqs = [_req(k, 20, 2 + k % 3, arrival=0.002 * k) for k in range(8)]
    st = eng.run(reqs, duration=None, drain=True)
    assert st["completed_requests"] == 8 and st["queued_requests"] == 0
    assert st["frame_latency_ms_p50"] is not None and st["frames"] == sum(r.frames for r in reqs)
    assert st["throughput"] > 0


def test_serving_request_mix_shapes():
    reqs = scene.serving_requests(rate=200.0, duration=0.2, seed=1, v_range=(1000, 5000), classes=4)
    assert len(reqs) > 10
    arr = [r.arrival for r in reqs]
    assert arr == sorted(arr) and arr[-1] <= 0.2
    for r in reqs:
        assert 30 <= r.frames <= 240
        assert 900 <= len(r.cloth.positions_world) <= 5500


class WorkClock:
    """Engine clock that advances only while a cohort's frame runs: by its
    work (vertex-substeps) over a fixed device rate."""

    def __init__(self, rate):
        self.t, self.rate = 0.0, rate

    def __call__(self):
        return self.t


class TimedBackend(FakeBackend):
    def __init__(self, clock):
        super().__init__()
        self.clock = clock
        self.max_resident = 0

    def wait(self, solver):
        live = [r for r, a in zip(solver.reqs, solver.active) if a]
        self.clock.t += sum(len(r.cloth.positions_world) * r.substeps for r in live) / self.clock.rate

    def step(self, solver, substeps, iterations):
        super().step(solver, substeps, iterations)


def test_latency_target_bounds_resident_work():
    """With a frame-latency target the engine keeps the resident work per
    tick within what the measured rate does in that time: 1,600-vertex
    requests at 10 substeps take 10 ms each at the fake device's rate, so a
    35 ms target keeps at most three resident and every frame within it,
    while all requests still complete in arrival order."""
    clock = WorkClock(rate=1.6e6)
    be = TimedBackend(clock)
    reqs = [_req(k, 40, 4) for k in range(9)]
    eng = ServingEngine(hbm_budget_bytes=1 << 40, backend=be, clock=clock, workers=0, frame_latency_ms=35.0,
                        rate_guess=1.6e6, max_admit_per_tick=64)
    for r in reqs:
        eng.submit(r)
    results, resident = [], []
    while not eng.idle():
        results += eng.tick()
        resident.append(eng.live_requests)
    assert max(resident) <= 3
    assert sorted(r.request_id for r in results) == list(range(9))
    lat = [x for r in results for x in r.frame_latency_ms]
    assert max(lat) <= 35.0 + 1e-6
    # without a target the memory budget alone admits everything at once
    clock2 = WorkClock(rate=1.6e6)
    eng2 = ServingEngine(hbm_budget_bytes=1 << 40, backend=TimedBackend(clock2), clock=clock2, workers=0)
    for r in [_req(k, 40, 4) for k in range(9)]:
        eng2.submit(r)
    eng2.tick()
    assert eng2.live_requests == 9


def test_latency_headroom_scales_the_admitted_work():
    """Admission keeps the resident work within `latency_headroom` of what
    the measured rate does in one target: 16,000 vertex-substeps per
    request at 1.6e6 per second, a 31 ms target holds 49,600 at full
    headroom (three requests) and 44,640 at the default 0.9 (two)."""
    for headroom, most in ((1.0, 3), (0.9, 2)):
        clock = WorkClock(rate=1.6e6)
        eng = ServingEngine(hbm_budget_bytes=1 << 40, backend=TimedBackend(clock), clock=clock, workers=0,
                            frame_latency_ms=31.0, rate_guess=1.6e6, max_admit_per_tick=64,
                            latency_headroom=headroom)
        for r in [_req(k, 40, 4) for k in range(6)]:
            eng.submit(r)
        resident = []
        results = []
        while not eng.idle():
            results += eng.tick()
            resident.append(eng.live_requests)
        assert max(resident) == most, (headroom, resident)
        assert sorted(r.request_id for r in results) == list(range(6))
