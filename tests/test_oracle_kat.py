"""The CPU oracle against the reference's known-answer smoke cases."""
import numpy as np
import pytest

import kat_cases


@pytest.mark.parametrize("make", kat_cases.ALL, ids=lambda f: f.__name__)
def test_oracle_known_answers(make, oracle_lib):
    case, run = make()
    solver = oracle_lib.OracleSolver(case.cfg, case.mesh, case.keep, case.pins)
    out = run(solver)
    assert np.isfinite(out).all()


def test_oracle_self_counters(oracle_lib):
    """abi41_smoke.cpp:292-300: the self-collision case records contacts and
    candidates in the counters."""
    case, run = kat_cases.self_vv()
    solver = oracle_lib.OracleSolver(case.cfg, case.mesh, case.keep, case.pins)
    run(solver)
    counts = solver.read_buffer(13, np.uint64, 38)
    assert counts[0] + counts[1] > 0  # soft + exact-impulse contacts
    assert counts[9] > 0  # candidates


def test_oracle_hard_stretch_known_answers(oracle_lib):
    """abi41_smoke.cpp:599-876 (PCG hard stretch) on the oracle."""
    kat_cases.hard_stretch_suite(lambda c: oracle_lib.OracleSolver(c.cfg, c.mesh, c.keep, c.pins))
