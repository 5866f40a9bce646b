"""Dynamic colliders on the GPU against the oracle: plain triangles
(unsigned response), indexed closed meshes (signed response with the
inside-only passes), particles, their spatial hashes (>= 64 triangles /
>= 128 particles) and brute-force paths, the large-triangle list, motion
continuity across uploads, and a batch whose cloths each equal their solo
run.  Every case moves its colliders every frame; positions must equal the
oracle's bit for bit after each frame (so they also meet the 1e-4 x cloth
extent tolerance), and the dynamic-collider counters must match."""
import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.native import NativeXpbdBatch, NativeXpbdSolver

pytestmark = pytest.mark.gpu

# counter slots: exact contacts, particle candidates / contacts, triangle
# pairs, friction corrections, triangle candidates, AABB rejects
DYN_SLOTS = [1, 4, 5, 7, 33, 34, 37]


def _sphere_center(f, radius=0.2, x=0.1):
    return np.array([x, 0.0, -(radius + 0.06) + 0.006 * f], np.float32)


def _sphere(f, sub=3, radius=0.2, x=0.1):
    """Icosphere rising 0.36 m/s; at 3 subdivisions (1280 triangles, ~2.6 cm
    edges) its triangles span few 2 cm hash cells."""
    v, i = scene.icosphere(_sphere_center(f, radius, x), radius, sub)
    return (v, i, False)


def _ramp(f, n=8):
    return scene.ramp_triangles((0.0, 0.05, -0.12 + 0.004 * f), 1.3, n, 0.25)


def _particles(f, count=300):
    p, r = scene.particle_stream(count, (0.0, 0.0, -0.1), 0.45, 0.04, seed=7)
    p = p + np.float32(0.003 * f) * np.array([0.3, -0.2, 1.0], np.float32)
    return (p, r)


def _floor_mesh(f):
    """A coarse icosphere (0.3 m, 320 triangles of ~8 cm) plus two 2 m
    triangles (a floor quad): all span more than 64 hash cells of 2 cm and
    go to the large list."""
    v, i, _ = _sphere(f, sub=2, radius=0.3)
    z = -0.25 + 0.004 * f
    q = np.array([[-1, -1, z], [1, -1, z], [1, 1, z], [-1, 1, z]], np.float32)
    qi = np.array([[0, 1, 2], [0, 2, 3]], np.int32) + len(v)
    return (np.concatenate([v, q]), np.concatenate([i, qi]), False)


CASES = {
    "ramp_hashed": lambda f: {"triangles": _ramp(f)},
    "ramp_brute": lambda f: {"triangles": _ramp(f, n=4)},
    "sphere_signed_hashed": lambda f: {"indexed": _sphere(f)},
    "sphere_signed_brute": lambda f: {"indexed": _sphere(f, sub=0, radius=0.3)},
    "particles_hashed": lambda f: {"particles": _particles(f)},
    "particles_brute": lambda f: {"particles": _particles(f, count=40)},
    "signed_with_particles": lambda f: {"indexed": _sphere(f, x=0.25), "particles": _particles(f, 160)},
    "unsigned_with_particles": lambda f: {"triangles": _ramp(f), "particles": _particles(f, 200)},
    "large_triangles": lambda f: {"indexed": _floor_mesh(f)},
}


def _pair(sc, oracle_lib):
    gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    ora = oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    return gpu, ora


def _run(name, frames, oracle_lib, n=24):
    sc = scene.dynamic_scene(n, frames)
    gpu, ora = _pair(sc, oracle_lib)
    totals = np.zeros(38, np.uint64)
    for f in range(frames):
        kw = CASES[name](f)
        gpu.update_dynamic_colliders(**kw)
        ora.update_dynamic_colliders(**kw)
        gpu.step(sc.substeps, sc.iterations, diagnostics=True, synchronize=True)
        ora.step(sc.substeps, sc.iterations)
        pg, po = gpu.download_positions(), ora.download_positions()
        assert np.isfinite(pg).all()
        err = float(np.abs(pg - po).max())
        assert err <= 1e-4 * sc.extent, (name, f, err)
        assert np.array_equal(pg, po), (name, f, err)
        cg = gpu.read_buffer(13, np.uint64, 38)
        co = ora.read_buffer(13, np.uint64, 38)
        assert np.array_equal(cg[DYN_SLOTS], co[DYN_SLOTS]), (name, f, cg[DYN_SLOTS], co[DYN_SLOTS])
        totals += cg
    return gpu, ora, totals, sc


@pytest.mark.parametrize("name", sorted(CASES))
def test_dynamic_matches_oracle(name, gpu_lib, oracle_lib):
    gpu, ora, totals, _ = _run(name, 14, oracle_lib)
    # the colliders reach the cloth: contacts were resolved
    assert totals[1] > 0, (name, totals[DYN_SLOTS])
    d = gpu.diagnostics()
    kw = CASES[name](13)
    if "triangles" in kw:
        assert d["dynamic_triangle_count"] == len(kw["triangles"])
        assert d["dynamic_triangle_candidate_count"] == int(gpu.read_buffer(13, np.uint64, 38)[34])
    if "indexed" in kw:
        assert d["dynamic_triangle_count"] == len(kw["indexed"][1])
    if "particles" in kw:
        assert d["dynamic_particle_count"] == len(kw["particles"][0])
    info = ora.dynamic_info()
    hashed = ("triangles" in kw and len(kw["triangles"]) >= 64) or ("indexed" in kw and len(kw["indexed"][1]) >= 64)
    assert info["tri_hashed"] == hashed
    assert d["dynamic_triangle_max_bucket_occupancy"] == info["max_occupancy"]
    assert (info["max_occupancy"] > 0) == (hashed and info["large"] < info["triangles"])
    assert d["dynamic_triangle_large_primitive_count"] == info["large"]
    if name == "large_triangles":
        assert info["large"] >= 2
    if name == "sphere_signed_hashed":
        assert info["large"] < info["triangles"] // 4


def test_dynamic_clear_and_topology_change(gpu_lib, oracle_lib):
    """Clearing a kind (empty arrays) and re-uploading with a topology change
    (no collider velocity on that frame) stay equal to the oracle."""
    sc = scene.dynamic_scene(20, 10)
    gpu, ora = _pair(sc, oracle_lib)
    for f in range(10):
        v, i, _ = _sphere(f)
        if f == 4:
            kw = {"indexed": (np.empty((0, 3), np.float32), np.empty((0, 3), np.int32), False),
                  "particles": _particles(f, 150)}
        elif f == 6:
            kw = {"indexed": (v, i[::-1].copy(), True), "particles": (np.empty((0, 3), np.float32), np.empty(0, np.float32))}
        else:
            kw = {"indexed": (v, i, False)}
        gpu.update_dynamic_colliders(**kw)
        ora.update_dynamic_colliders(**kw)
        gpu.step(sc.substeps, sc.iterations, diagnostics=False, synchronize=True)
        ora.step(sc.substeps, sc.iterations)
        pg, po = gpu.download_positions(), ora.download_positions()
        assert np.array_equal(pg, po), (f, float(np.abs(pg - po).max()))


def test_dynamic_signed_keeps_cloth_outside(gpu_lib, oracle_lib):
    """A closed sphere rising into a falling cloth: after the signed passes no
    cloth vertex is left inside the sphere by more than the thickness."""
    gpu, _, _, _ = _run("sphere_signed_hashed", 20, oracle_lib, n=20)
    p = gpu.download_positions()
    d = np.linalg.norm(p - _sphere_center(19), axis=1)
    # the icosphere's flat faces lie inside the sphere radius by < 0.5 %
    assert d.min() > 0.2 * 0.995 - 0.01, d.min()


@pytest.mark.parametrize("graphs", [True, False])
def test_dynamic_batch_alone_equals_mix(graphs, gpu_lib):
    """Three cloths in one batch (signed sphere; ramp + particles; none) each
    equal the same cloth in its own solver, with graph capture on and off."""
    scs = [scene.dynamic_scene(n, 8) for n in (16, 20, 12)]
    batch = NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs])
    batch.set_graph_capture(graphs)
    solo = [NativeXpbdSolver(s.cloth, s.options, s.static_triangles) for s in scs]
    for f in range(8):
        kws = [{"indexed": _sphere(f)}, {"triangles": _ramp(f), "particles": _particles(f, 200)}, {}]
        for k, kw in enumerate(kws):
            if kw:
                batch.update_cloth_dynamic_colliders(k, **kw)
                solo[k].update_dynamic_colliders(**kw)
        batch.step(10, 2, diagnostics=False, synchronize=True)
        for k, s in enumerate(solo):
            s.step(10, 2, diagnostics=False, synchronize=True)
            assert np.array_equal(batch.download_cloth_positions(k), s.download_positions()), (f, k)
