"""The oracle's shared dynamic scene: source filtering (a cloth never collides
with its own source; mode 2 keeps only lower layers), mode 0 keeps the
cloth's own colliders, and particle overflow counts."""
import numpy as np

from xpbd_gb300 import scene


def _cloth(oracle_lib, n=16):
    sc = scene.dynamic_scene(n, 6)
    return sc, oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)


def _floor(z=-0.02, cells=8):
    return scene.ramp_triangles((0.0, 0.0, z), 1.4, cells, 0.0)


def _run(oracle_lib, src, layer, mode, tri_src, tri_layer, frames=10):
    sc, s = _cloth(oracle_lib)
    g = oracle_lib.OracleScene()
    rows = _floor()
    g.update(triangles=(rows, np.full(len(rows), tri_src, np.int32), np.full(len(rows), tri_layer, np.int32)),
             margin=0.005, thickness=0.002)
    s.attach_global_scene(g, src, layer, mode)
    for _ in range(frames):
        s.step(sc.substeps, sc.iterations)
    p = s.download_positions().copy()
    s.clear_global_scene()
    g.close()
    return p


def test_scene_floor_catches_the_cloth(oracle_lib):
    caught = _run(oracle_lib, 1, 0, 1, tri_src=2, tri_layer=0)
    assert caught[:, 2].min() > -0.02 - 0.01


def test_own_source_is_skipped(oracle_lib):
    own = _run(oracle_lib, 2, 0, 1, tri_src=2, tri_layer=0)
    assert own[:, 2].min() < -0.06  # fell through its own source's floor


def test_layers(oracle_lib):
    lower = _run(oracle_lib, 1, 3, 2, tri_src=2, tri_layer=1)
    higher = _run(oracle_lib, 1, 3, 2, tri_src=2, tri_layer=5)
    assert lower[:, 2].min() > -0.03 and higher[:, 2].min() < -0.06


def test_mode_zero_keeps_own_colliders(oracle_lib):
    sc, s = _cloth(oracle_lib)
    g = oracle_lib.OracleScene()
    rows = _floor()
    g.update(triangles=(rows, np.full(len(rows), 2, np.int32), np.zeros(len(rows), np.int32)), margin=0.005)
    s.attach_global_scene(g, 1, 0, 0)
    for _ in range(10):
        s.step(sc.substeps, sc.iterations)
    assert s.download_positions()[:, 2].min() < -0.06  # the scene is not read in mode 0
    s.clear_global_scene()


def test_particle_overflow_counted(oracle_lib):
    g = oracle_lib.OracleScene()
    n = 200
    pos = np.zeros((n, 3), np.float32)  # all in one cell: one bucket of 200
    g.update(particles=(pos, None, np.full(n, 0.01, np.float32), np.ones(n, np.int32), np.zeros(n, np.int32)), margin=0.005)
    assert g.overflow() == n - 16
