"""Properties of the oracle that the GPU parity tests rely on."""
import numpy as np

from xpbd_gb300 import scene


def _drop(oracle_lib, n=40, mode=2):
    sc = scene.drop_scene(n, 2, seed=1, self_mode=mode)
    return sc, oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)


def test_oracle_is_thread_count_independent(oracle_lib):
    outs = []
    for threads in (1, 4):
        oracle_lib.set_threads(threads)
        sc, s = _drop(oracle_lib)
        for _ in range(3):
            s.step(sc.substeps, sc.iterations)
        outs.append(s.download_positions().copy())
    oracle_lib.set_threads(0)
    assert np.array_equal(outs[0], outs[1])


def test_hash_structures_are_consistent(oracle_lib):
    sc, s = _drop(oracle_lib, 40)
    s.build_self_structures()
    nvb, ntb, neb, vh, th, eh = s.hash_info()
    assert vh == 1 and th == 1 and eh == 1
    V = len(sc.cloth.positions_world)
    cells = s.read_buffer(3, np.int32, 4 * V).reshape(V, 4)
    start = s.read_buffer(4, np.int32, nvb + 1)
    ent = s.read_buffer(5, np.int32, V)
    assert start[0] == 0 and start[-1] == V and np.all(np.diff(start) >= 0)
    # every vertex listed once, in its own bucket, buckets in increasing id order
    assert np.array_equal(np.sort(ent), np.arange(V))
    for b in np.flatnonzero(np.diff(start)):
        members = ent[start[b]:start[b + 1]]
        assert np.all(np.diff(members) > 0)
        assert np.all(cells[members, 3] == b)
    # bucket ids are the Teschner hash of the cells
    c = cells[:, :3].astype(np.int64).astype(np.uint32)
    h = (c[:, 0] * np.uint32(73856093)) ^ (c[:, 1] * np.uint32(19349663)) ^ (c[:, 2] * np.uint32(83492791))
    assert np.array_equal((h & np.uint32(nvb - 1)).astype(np.int32), cells[:, 3])
    # neighbour lists reference distinct other vertices
    cnt = s.read_buffer(10, np.int32, V)
    idx = s.read_buffer(11, np.int32, V * 32).reshape(V, 32)
    for v in np.flatnonzero(cnt)[:200]:
        row = idx[v, :cnt[v]]
        assert v not in row and len(set(row.tolist())) == len(row)


def test_plain_cloth_falls_and_pins_hold(oracle_lib):
    sc = scene.plain_grid_scene(32, 10)
    s = oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    for _ in range(10):
        s.step(sc.substeps, sc.iterations)
    p = s.download_positions()
    assert np.isfinite(p).all()
    pins = sc.cloth.pin_indices
    assert np.abs(p[pins] - sc.cloth.pin_targets_world).max() <= 1e-6
    assert p[:, 2].min() < -0.05
