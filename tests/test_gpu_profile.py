"""The profiled frame behind bench.py's per-kernel table and roofline: it
advances the solver like a stepped frame (same positions as the oracle),
times every kernel kind it launches, and its work counters describe the
frame's query work and the size of its hash builds."""
import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.native import NativeXpbdSolver

pytestmark = pytest.mark.gpu


def test_profiled_frame_counters(gpu_lib, oracle_lib):
    sc = scene.drop_scene(40, 4, seed=2)
    gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    ora = oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    prof = gpu.profile_frame(sc.substeps, sc.iterations)
    ora.step(sc.substeps, sc.iterations)
    assert np.array_equal(gpu.download_positions(), ora.download_positions())
    assert set(prof) <= set(NativeXpbdSolver.KERNEL_KINDS)
    for kind in ("predict", "vertex_hash", "triangle_hash", "edge_hash", "neighbors", "edge_edge", "self_apply"):
        ms, n = prof[kind]
        assert n > 0 and ms > 0.0, kind
    c = gpu.profile_counters()
    E, T = len(sc.cloth.edges), len(sc.cloth.triangles)
    assert c["edge_hashed"] == E and c["tri_hashed"] == T
    # every primitive enters at least the one cell of its box, at most 64
    assert E <= c["edge_entries"] <= 64 * E and T <= c["tri_entries"] <= 64 * T
    assert c["edge_buckets"] >= 4 * E and c["tri_buckets"] >= 4 * T
    assert c["ee_items"] > 0 and c["ee_slots"] >= c["ee_items"]
