"""The reference's contact-group probe cases (tests/kat_probe_cases.py) on
the GPU: positions and all 38 counters equal the oracle's after every step,
for the analytic ground / wall / sphere / corner contacts, the static SDF
plane and the self VV pair."""
import numpy as np
import pytest

import kat_probe_cases as kp
from xpbd_gb300.native import NativeXpbdSolver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", kp.KINDS)
def test_probe_case_matches_oracle(kind, gpu_lib, oracle_lib):
    cl, opts, static, penetration, _ = kp.analytic(kind)
    gpu = NativeXpbdSolver(cl, opts, static)
    ora = oracle_lib.OracleSolver.from_scene(cl, opts, static)
    for step in range(kp.STEPS):
        gpu.step(kp.SUBSTEPS, kp.ITERATIONS, diagnostics=True, synchronize=True)
        ora.step(kp.SUBSTEPS, kp.ITERATIONS)
        assert np.array_equal(gpu.download_positions(), ora.download_positions()), (kind, step)
        assert np.array_equal(gpu.read_buffer(13, np.uint64, 38), ora.read_buffer(13, np.uint64, 38)), (kind, step)
    assert penetration(gpu.download_positions()) < 0.01
    if kind == "static_sdf":
        assert gpu.diagnostics()["static_sdf_contact_count"] > 0


def test_probe_self_vv_matches_oracle(gpu_lib, oracle_lib):
    cl, opts, close = kp.self_vv_line()
    gpu = NativeXpbdSolver(cl, opts, kp.NO_STATIC)
    ora = oracle_lib.OracleSolver.from_scene(cl, opts, kp.NO_STATIC)
    gpu.update_positions(close)
    ora.update_positions(close)
    for _ in range(2):
        gpu.step(1, 6, diagnostics=True, synchronize=True)
        ora.step(1, 6)
        assert np.array_equal(gpu.download_positions(), ora.download_positions())
        assert np.array_equal(gpu.read_buffer(13, np.uint64, 38), ora.read_buffer(13, np.uint64, 38))
    out = gpu.download_positions()
    assert float(np.linalg.norm(out[-1] - out[0])) > 0.03


@pytest.mark.parametrize("case", sorted(kp.SMOKES))
def test_self_collision_smoke(case, gpu_lib, oracle_lib):
    """tools/abi41_self_collision_smoke.py's pass conditions on the GPU
    (contacts and candidates reported, a positive smoothed delta, the pair
    separated by more than 1e-4), and GPU == oracle bit for bit."""
    cl, close, measure = kp.SMOKES[case]()
    opts = kp.smoke_options()
    gpu = NativeXpbdSolver(cl, opts, kp.NO_STATIC)
    ora = oracle_lib.OracleSolver.from_scene(cl, opts, kp.NO_STATIC)
    gpu.update_positions(close)
    ora.update_positions(close)
    gpu.step(1, 6, diagnostics=True, synchronize=True)
    ora.step(1, 6)
    out = gpu.download_positions().copy()
    assert np.array_equal(out, ora.download_positions())
    assert np.array_equal(gpu.read_buffer(13, np.uint64, 38), ora.read_buffer(13, np.uint64, 38))
    d = gpu.diagnostics()
    assert np.isfinite(out).all() and d["finite_flag"]
    if case == "vv":
        assert d["abi41_soft_contact_count"] + d["abi41_exact_impulse_contact_count"] > 0
        assert d["fast_soft_repulsion_candidates"] > 0
    elif case == "vt":
        assert d["abi41_soft_contact_count"] > 0 and d["fast_soft_repulsion_candidates"] > 0
    else:
        assert d["abi41_edge_edge_contact_count"] > 0 and d["resolved_contacts"] > 0
    assert d["abi41_max_smoothed_delta"] > 0.0
    assert measure(out) > measure(close) + 1.0e-4
