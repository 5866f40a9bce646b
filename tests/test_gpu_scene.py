"""Shared dynamic scene (cross-cloth collision) on the GPU against the
oracle: triangles and particles of several sources with layers, moving every
frame; a single cloth and every cloth of a batch attached with their own
source filters (all-but-own and lower-layers modes), mode 0, detaching, and
destroying a scene that is still attached.  Positions and the dynamic
counters must equal the oracle's bit for bit."""
import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.native import GlobalDynamicScene, NativeXpbdBatch, NativeXpbdSolver

pytestmark = pytest.mark.gpu
DYN_SLOTS = [1, 4, 5, 7, 33, 34, 37]


def _scene_data(f):
    """Source 1: a floor under cloth 0 (layer 0); source 2: a tilted ramp
    (layer 2); source 3: particles rising (layer 1)."""
    floor = scene.ramp_triangles((0.0, 0.0, -0.02 + 0.002 * f), 1.4, 8, 0.0)
    ramp = scene.ramp_triangles((0.2, 0.0, -0.05 + 0.004 * f), 1.2, 6, 0.3)
    rows = np.concatenate([floor, ramp])
    src = np.concatenate([np.full(len(floor), 1), np.full(len(ramp), 2)]).astype(np.int32)
    layer = np.concatenate([np.zeros(len(floor)), np.full(len(ramp), 2)]).astype(np.int32)
    p, r = scene.particle_stream(180, (0.0, 0.0, -0.08), 0.45, 0.03, seed=9)
    prev = p + np.float32(0.003 * f)
    cur = p + np.float32(0.003 * (f + 1))
    return {"triangles": (rows, src, layer),
            "particles": (cur, prev, r, np.full(len(p), 3, np.int32), np.ones(len(p), np.int32)),
            "margin": 0.005, "thickness": 0.002}


@pytest.mark.parametrize("src,layer,mode", [(1, 0, 1), (2, 0, 1), (9, 2, 2), (9, 1, 2), (1, 0, 0)],
                         ids=["skip-floor", "skip-ramp", "layers-below-2", "layers-below-1", "mode0"])
def test_scene_single_cloth(src, layer, mode, gpu_lib, oracle_lib):
    sc = scene.dynamic_scene(20, 10)
    gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    ora = oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    gs, os_ = GlobalDynamicScene(), oracle_lib.OracleScene()
    gpu.attach_global_scene(gs, src, layer, mode)
    ora.attach_global_scene(os_, src, layer, mode)
    contacts = 0
    for f in range(10):
        data = _scene_data(f)
        gs.update(**data)
        os_.update(**data)
        gpu.step(10, 2, diagnostics=True, synchronize=True)
        ora.step(10, 2)
        pg, po = gpu.download_positions(), ora.download_positions()
        assert np.array_equal(pg, po), (f, float(np.abs(pg - po).max()))
        cg, co = gpu.read_buffer(13, np.uint64, 38), ora.read_buffer(13, np.uint64, 38)
        assert np.array_equal(cg[DYN_SLOTS], co[DYN_SLOTS]), (f, cg[DYN_SLOTS], co[DYN_SLOTS])
        contacts += int(cg[1])
    d = gpu.diagnostics()
    if mode != 0:
        assert contacts > 0
        assert d["global_dynamic_triangle_count"] == len(data["triangles"][0])
        assert d["global_dynamic_particle_count"] == len(data["particles"][0])
        assert d["global_dynamic_hash_overflow"] == os_.overflow()
    else:
        assert contacts == 0 and d["global_dynamic_triangle_count"] == 0
    ora.clear_global_scene()


def test_scene_shared_by_a_batch(gpu_lib, oracle_lib):
    """Three cloths of one batch read one scene, each skipping its own source."""
    scs = [scene.dynamic_scene(n, 8) for n in (16, 20, 12)]
    filters = [(1, 0, 1), (3, 0, 1), (9, 2, 2)]
    batch = NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs])
    oras = [oracle_lib.OracleSolver.from_scene(s.cloth, s.options, s.static_triangles) for s in scs]
    gs, os_ = GlobalDynamicScene(), oracle_lib.OracleScene()
    for k, (src, layer, mode) in enumerate(filters):
        batch.attach_cloth_global_scene(k, gs, src, layer, mode)
        oras[k].attach_global_scene(os_, src, layer, mode)
    for f in range(8):
        data = _scene_data(f)
        gs.update(**data)
        os_.update(**data)
        batch.step(10, 2, diagnostics=False, synchronize=True)
        for k, o in enumerate(oras):
            o.step(10, 2)
            assert np.array_equal(batch.download_cloth_positions(k), o.download_positions()), (f, k)
    # detaching one cloth returns it to its own (empty) colliders
    batch.clear_cloth_global_scene(1)
    oras[1].clear_global_scene()
    batch.step(10, 2, diagnostics=False, synchronize=True)
    for k, o in enumerate(oras):
        o.step(10, 2)
        assert np.array_equal(batch.download_cloth_positions(k), o.download_positions()), ("detached", k)
    for o in oras:
        o.clear_global_scene()


def test_destroying_an_attached_scene_detaches(gpu_lib, oracle_lib):
    sc = scene.dynamic_scene(16, 6)
    gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    ora = oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    gs = GlobalDynamicScene()
    gs.update(**_scene_data(0))
    gpu.attach_global_scene(gs, 2, 0, 1)
    gs.close()  # the solver stops reading it
    for _ in range(3):
        gpu.step(10, 2, diagnostics=False, synchronize=True)
        ora.step(10, 2)
        assert np.array_equal(gpu.download_positions(), ora.download_positions())


def test_scene_validation(gpu_lib):
    gs = GlobalDynamicScene()
    from xpbd_gb300.native import NativeSolverError, scene_inputs

    fi, keep = scene_inputs()
    fi.triangle_count = 3  # no arrays
    import ctypes

    assert gs._lib.ssbl_update_global_dynamic_scene(gs.handle, ctypes.byref(fi)) == 0
    from xpbd_gb300.native import _last_error

    assert "global dynamic triangle arrays are incomplete" in _last_error(gs._lib)
    fi.triangle_count = 0
    fi.particle_count = 2
    assert gs._lib.ssbl_update_global_dynamic_scene(gs.handle, ctypes.byref(fi)) == 0
    assert "global dynamic particle arrays are incomplete" in _last_error(gs._lib)
