"""Launch configuration and autotuner on the GPU: no block size or tile
choice changes a result (positions and counters stay equal to the oracle's
bit for bit), the autotuner leaves the solver's state as it found it, and
invalid values are refused."""
import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.native import NativeSolverError, NativeXpbdBatch, NativeXpbdSolver

pytestmark = pytest.mark.gpu

CONFIGS = [
    {"vertex_block": 64, "hash_block": 128, "prim_lanes": 4, "warp_block": 128, "query_block": 64, "group_lanes": 4,
     "group_block": 128, "dynamic_block": 64, "fast_ee_form": 8, "tri_lanes": 1, "neighbor_lanes": 1},
    {"vertex_block": 256, "hash_block": 256, "prim_lanes": 16, "warp_block": 256, "query_block": 256, "group_lanes": 16,
     "group_block": 256, "dynamic_block": 256, "fast_ee_form": 32, "tri_lanes": 16, "neighbor_lanes": 32},
    {"vertex_block": 96, "query_block": 160, "warp_block": 32},
]


def _mix():
    scs = scene.batched_scenes(3, seed=5, frames=4, side_range=(12, 24))
    sc = scene.drop_scene(14, 4, seed=2)
    sc.options.max_self_collision_neighbors = 6  # strict group queries
    scs.append(sc)
    scs.append(scene.drop_scene(12, 4, seed=3, self_mode=1))
    return scs


@pytest.mark.parametrize("cfg", range(len(CONFIGS)))
def test_launch_config_keeps_results(cfg, gpu_lib, oracle_lib):
    scs = _mix()
    batch = NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs])
    batch.set_launch_config(CONFIGS[cfg])
    got = batch.launch_config()
    for k, v in CONFIGS[cfg].items():
        assert got[k] == v
    oras = [oracle_lib.OracleSolver.from_scene(s.cloth, s.options, s.static_triangles) for s in scs]
    for frame in range(3):
        batch.step(10, 2, diagnostics=False, synchronize=True)
        for k, o in enumerate(oras):
            o.step(10, 2)
            assert np.array_equal(batch.download_cloth_positions(k), o.download_positions()), (cfg, frame, k)


def test_dynamic_block_keeps_results(gpu_lib, oracle_lib):
    sc = scene.dynamic_scene(16, 4)
    gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    ora = oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    gpu.set_launch_config({"dynamic_block": 32})
    for f in range(4):
        v, i = scene.icosphere((0.0, 0.0, -0.26 + 0.006 * f), 0.2, 3)
        for s in (gpu, ora):
            s.update_dynamic_colliders(indexed=(v, i, False))
        gpu.step(10, 2, diagnostics=False, synchronize=True)
        ora.step(10, 2)
        assert np.array_equal(gpu.download_positions(), ora.download_positions()), f


def test_autotune_restores_state_and_keeps_results(gpu_lib, oracle_lib, tmp_path, monkeypatch):
    monkeypatch.setenv("XPBD_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    scs = _mix()
    batch = NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs])
    oras = [oracle_lib.OracleSolver.from_scene(s.cloth, s.options, s.static_triangles) for s in scs]
    batch.step(10, 2, diagnostics=False, synchronize=True)
    for o in oras:
        o.step(10, 2)
    before = batch.download_positions().copy()
    r = batch.autotune(10, 2, rounds=1)
    assert not r["cached"] and r["tuned_ms"] <= r["default_ms"] and set(r["config"]) == set(batch.LAUNCH_SLOTS)
    assert np.array_equal(batch.download_positions(), before)
    for frame in range(2):
        batch.step(10, 2, diagnostics=False, synchronize=True)
        for k, o in enumerate(oras):
            o.step(10, 2)
            assert np.array_equal(batch.download_cloth_positions(k), o.download_positions()), (frame, k)
    # a second solver of the same workload takes the cached configuration
    again = NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs])
    r2 = again.autotune(10, 2, rounds=1)
    assert r2["cached"] and again.launch_config() == r["config"]


@pytest.mark.parametrize("bad", [{"vertex_block": 512}, {"vertex_block": 100}, {"prim_lanes": 32}, {"group_lanes": 2},
                                 {"fast_ee_form": 16}])
def test_invalid_launch_config_is_refused(bad, gpu_lib):
    sc = scene.plain_grid_scene(8, 1)
    s = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    with pytest.raises(NativeSolverError, match="invalid launch configuration"):
        s.set_launch_config(bad)
