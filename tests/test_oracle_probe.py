"""The reference's contact-group probe cases (tests/kat_probe_cases.py) on
the oracle: every contact holds the vertex near the collider's margin
against a gravity that pushes it in, friction limits the sliding, and the
close VV pair is pushed apart."""
import numpy as np
import pytest

import kat_probe_cases as kp


def _run(oracle_lib, cl, opts, static):
    s = oracle_lib.OracleSolver.from_scene(cl, opts, static)
    for _ in range(kp.STEPS):
        s.step(kp.SUBSTEPS, kp.ITERATIONS)
    return s.download_positions().copy(), s.read_buffer(13, np.uint64, 38)


@pytest.mark.parametrize("kind", kp.KINDS)
def test_probe_contact_holds(kind, oracle_lib):
    cl, opts, static, penetration, tangent = kp.analytic(kind)
    out, _ = _run(oracle_lib, cl, opts, static)
    assert np.isfinite(out).all()
    # pushed into the collider for 28 frames, the vertex stays within 1 cm of
    # the 5 cm margin
    assert penetration(out) < 0.01, (kind, penetration(out))
    # where gravity presses the vertex into the collider, friction 4.0 keeps
    # the tangential drift well under free sliding (the sphere case's gravity
    # has no component into the sphere, so nothing holds it there)
    if kind != "sphere":
        assert tangent(out) < 0.25 * kp.free_tangent(kind), (kind, tangent(out))


def test_probe_self_vv_pushes_apart(oracle_lib):
    cl, opts, close = kp.self_vv_line()
    s = oracle_lib.OracleSolver.from_scene(cl, opts, kp.NO_STATIC)
    s.update_positions(close)
    s.step(1, 6)
    out = s.download_positions().copy()
    s.step(1, 6)
    follow = s.download_positions().copy()
    gap0 = float(np.linalg.norm(close[-1] - close[0]))
    gap1 = float(np.linalg.norm(out[-1] - out[0]))
    gap2 = float(np.linalg.norm(follow[-1] - follow[0]))
    assert np.isfinite(out).all() and np.isfinite(follow).all()
    assert gap1 > gap0  # the pair was separated
    assert gap2 >= gap1 - 1e-6  # and does not fall back


@pytest.mark.parametrize("case", sorted(kp.SMOKES))
def test_self_collision_smoke_oracle(case, oracle_lib):
    """tools/abi41_self_collision_smoke.py's conditions on the oracle: the
    pair separates by more than 1e-4 and contacts are counted (counter slots:
    0 soft, 1 exact impulse, 2 edge-edge, 9 self candidates)."""
    cl, close, measure = kp.SMOKES[case]()
    s = oracle_lib.OracleSolver.from_scene(cl, kp.smoke_options(), kp.NO_STATIC)
    s.update_positions(close)
    s.step(1, 6)
    out = s.download_positions().copy()
    c = s.read_buffer(13, np.uint64, 38)
    assert np.isfinite(out).all()
    assert measure(out) > measure(close) + 1.0e-4
    contacts = {"vv": int(c[0]) + int(c[1]), "vt": int(c[0]), "ee": int(c[2])}[case]
    assert contacts > 0 and (case == "ee" or int(c[9]) > 0)
