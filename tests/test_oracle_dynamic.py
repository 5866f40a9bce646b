"""Properties of the oracle's dynamic colliders that the GPU parity tests
rely on: the triangle hash finds the same contacts as the brute-force walk,
the threads do not change the result, signed contacts keep the cloth out of
a closed mesh, and the upload validation matches the reference's messages."""
import numpy as np
import pytest

from xpbd_gb300 import scene


def _cloth(oracle_lib, n=20):
    sc = scene.dynamic_scene(n, 8)
    return sc, oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)


def _flat(f, cells):
    return scene.ramp_triangles((0.0, 0.0, -0.06 + 0.004 * f), 1.4, cells, 0.0)


def test_hashed_triangles_find_the_brute_force_contacts(oracle_lib):
    """A flat moving floor as 128 triangles (hashed) and as 8 (brute force):
    the unsigned response depends on the deepest contact only, which both
    find; closest points on different triangulations of one plane differ in
    the last bits only."""
    runs = []
    for cells in (8, 2):
        sc, s = _cloth(oracle_lib)
        for f in range(8):
            s.update_dynamic_colliders(triangles=_flat(f, cells))
            s.step(sc.substeps, sc.iterations)
        runs.append((s.download_positions().copy(), s.dynamic_info()))
    (a, ia), (b, ib) = runs
    assert ia["tri_hashed"] and not ib["tri_hashed"]
    assert np.abs(a - b).max() < 2e-5
    # the floor caught the cloth
    assert a[:, 2].min() > -0.06 - 0.01


def test_dynamic_oracle_is_thread_count_independent(oracle_lib):
    outs = []
    for threads in (1, 4):
        oracle_lib.set_threads(threads)
        sc, s = _cloth(oracle_lib)
        for f in range(6):
            v, i = scene.icosphere((0.0, 0.0, -0.26 + 0.006 * f), 0.2, 3)
            p, r = scene.particle_stream(200, (0.0, 0.0, -0.1), 0.45, 0.04, seed=1)
            s.update_dynamic_colliders(indexed=(v, i, False), particles=(p + 0.003 * f, r))
            s.step(sc.substeps, sc.iterations)
        outs.append(s.download_positions().copy())
    oracle_lib.set_threads(0)
    assert np.array_equal(outs[0], outs[1])


def test_signed_mesh_keeps_cloth_outside(oracle_lib):
    sc, s = _cloth(oracle_lib, 24)
    for f in range(20):
        v, i = scene.icosphere((0.1, 0.0, -0.26 + 0.006 * f), 0.2, 3)
        s.update_dynamic_colliders(indexed=(v, i, False))
        s.step(sc.substeps, sc.iterations)
    p = s.download_positions()
    d = np.linalg.norm(p - np.array([0.1, 0.0, -0.26 + 0.006 * 19]), axis=1)
    assert d.min() > 0.2 * 0.995 - 0.01
    # the sphere lifted the cloth above where free fall would have left it
    assert p[:, 2].max() > 0.0


def test_particles_push_vertices_out(oracle_lib):
    sc, s = _cloth(oracle_lib, 16)
    p, r = scene.particle_stream(300, (0.0, 0.0, -0.05), 0.45, 0.04, seed=3)
    for f in range(10):
        s.update_dynamic_colliders(particles=(p, r))
        s.step(sc.substeps, sc.iterations)
    info = s.dynamic_info()
    assert info["par_hashed"] and info["particles"] == 300
    c = s.read_buffer(13, np.uint64, 38)
    assert c[5] > 0  # particle contacts in the last frame


def test_upload_validation(oracle_lib):
    sc, s = _cloth(oracle_lib, 8)
    lib = s._lib
    assert lib.oracle_update_dynamic_triangles(s._h, None, 3) == 0
    assert "dynamic triangle data is required" in lib.oracle_last_error().decode()
    assert lib.oracle_update_dynamic_particles(s._h, None, None, 2) == 0
    assert "position/radius data is required" in lib.oracle_last_error().decode()
    assert lib.oracle_update_dynamic_indexed(s._h, None, 3, None, 1, 0) == 0
    assert "positions and indices are required" in lib.oracle_last_error().decode()
    # zero counts clear without data
    assert lib.oracle_update_dynamic_triangles(s._h, None, 0) == 1
    assert lib.oracle_update_dynamic_indexed(s._h, None, 0, None, 0, 0) == 1


@pytest.mark.parametrize("bad", [-1, 5])
def test_indexed_rows_outside_the_vertices_are_degenerate(oracle_lib, bad):
    """An index outside the vertex range gives a triangle at the origin
    (abi41.cu:3663-3684); the step stays finite."""
    sc, s = _cloth(oracle_lib, 8)
    v = np.array([[0, 0, -0.5], [1, 0, -0.5], [0, 1, -0.5]], np.float32)
    idx = np.array([[0, 1, 2], [0, 1, bad]], np.int32)
    s.update_dynamic_colliders(indexed=(v, idx, True))
    s.step(sc.substeps, sc.iterations)
    assert np.isfinite(s.download_positions()).all()
