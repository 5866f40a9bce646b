"""Serving form on the GPU: requests that arrive while others run are
admitted as memory frees up, share cohorts, and each result is bit-identical
to the same request run alone (and to the oracle)."""
import copy

import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.native import NativeXpbdSolver
from xpbd_gb300.serving import ServingEngine, estimate_device_bytes

pytestmark = pytest.mark.gpu


def _mix():
    reqs = scene.serving_requests(rate=400.0, duration=1.0, seed=5, v_range=(150, 900), horizon=(2, 6), classes=5,
                                  max_requests=9)
    for k, r in enumerate(reqs):
        r.arrival = 0.0 if k < 4 else 0.05 * k  # some arrive while the first ones run
    return reqs


def test_result_same_alone_and_in_mix(gpu_lib, oracle_lib):
    reqs = _mix()
    budget = sum(sorted(estimate_device_bytes(r) for r in reqs)[-3:])  # at most about three resident at once
    eng = ServingEngine(hbm_budget_bytes=budget, group_below=10_000)
    st = eng.run(reqs, duration=None, drain=True)
    eng.close()
    assert st["completed_requests"] == len(reqs)
    assert eng.used_bytes == 0 and st["peak_device_bytes"] <= budget
    by_id = {r.request_id: r for r in st["results"]}
    shared = 0
    for req in reqs:
        res = by_id[req.request_id]
        alone = NativeXpbdSolver(req.cloth, req.options, req.static_triangles)
        for _ in range(req.frames):
            alone.step(req.substeps, req.iterations, diagnostics=False, synchronize=True)
        assert np.array_equal(res.positions, alone.download_positions()), req.request_id
        assert len(res.frame_latency_ms) == req.frames
        alone.close()
    # and one request against the oracle
    req = reqs[0]
    ora = oracle_lib.OracleSolver.from_scene(req.cloth, req.options, req.static_triangles)
    for _ in range(req.frames):
        ora.step(req.substeps, req.iterations)
    assert np.array_equal(by_id[req.request_id].positions, ora.download_positions())


def test_memory_estimate_covers_allocation(gpu_lib):
    reqs = _mix()[:5]
    # one request with the hard-stretch CG buffers
    hard = copy.deepcopy(reqs[0])
    hard.options.stretch_optimization_enabled = True
    hard.options.stretch_optimization_strength = 1.0
    for r in reqs + [hard]:
        s = NativeXpbdSolver(r.cloth, r.options, r.static_triangles)
        assert s.device_bytes() <= estimate_device_bytes(r), (len(r.cloth.positions_world), s.device_bytes())
        s.close()
