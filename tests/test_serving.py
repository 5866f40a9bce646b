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
