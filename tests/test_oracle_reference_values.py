"""The CPU oracle against values printed by the reference solver itself.

tests/golden/abi41_smoke_reference_gb300.txt holds the known-answer markers
that the reference's smoke program printed with the reference's own CUDA
solver on a GB300.  The oracle restates the same cases (tests/kat_cases.py);
here its results must equal the printed values at their printed precision
(5 decimals): the PCG hard-stretch case with and without a pinned end, and
the pin-weight case (weights 1.0 / 0.375 / 0.04).
"""
import os

import numpy as np
import pytest

import kat_cases
from test_gpu_ref_smoke import GOLDEN, marker_values


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return marker_values(f.read())


def _close(value, printed):
    return abs(float(value) - float(printed)) <= 5.0e-6 + 1e-7


def test_hard_stretch_matches_reference_values(oracle_lib, golden):
    g = golden["SSBL_ABI41_HARD_STRETCH_OK"]
    out = kat_cases.hard_stretch_suite(lambda c: oracle_lib.OracleSolver(c.cfg, c.mesh, c.keep, c.pins))
    off = np.linalg.norm(out["off"][1] - out["off"][0])
    on = np.linalg.norm(out["on"][1] - out["on"][0])
    both = np.linalg.norm(out["both_pinned"][1] - out["both_pinned"][0])
    assert _close(off, g["free.0"]), (off, g)
    assert _close(on, g["free.1"]), (on, g)
    assert _close(out["pinned"][1, 0], g["pinned_free"]), (out["pinned"], g)
    assert _close(both, g["both_pinned"]), (both, g)


def test_pin_weights_match_reference_values(oracle_lib, golden):
    g = golden["SSBL_ABI41_PIN_WEIGHT_OK"]
    case, run = kat_cases.pin_weights()
    out = run(oracle_lib.OracleSolver(case.cfg, case.mesh, case.keep, case.pins))
    for k, row in (("hard_y", 0), ("soft_y", 1), ("low_y", 2), ("free_y", 3)):
        assert _close(out[row, 1], g[k]), (k, out[row, 1], g[k])
