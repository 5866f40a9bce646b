"""Fused frames: a solver whose cloths each fit one block (at most 1024
vertices, no self collision, hard stretch or dynamic colliders) runs the
whole frame as one launch, a block per cloth, replaying the recorded
operations of the launched schedule.  Results equal the launched form and
the oracle bit for bit."""
import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.native import NativeXpbdBatch, NativeXpbdSolver

pytestmark = pytest.mark.gpu


def _small_mix():
    out = []
    for k, n in enumerate((32, 20, 31, 12)):
        sc = scene.plain_grid_scene(n, 6)
        out.append(sc)
    # tethers and gathered (uncoloured) bends
    sc = scene.plain_grid_scene(16, 6)
    w = np.zeros(len(sc.cloth.positions_world), np.float32)
    w[sc.cloth.pin_indices] = 1.0
    sc.cloth = scene.build_cloth(sc.cloth.positions_world, sc.cloth.triangles, 0.2, w, tether_slack=1.05)
    sc.cloth.bend_color_offsets = np.asarray([0], np.int32)
    sc.options.lra_compliance = 1e-6
    out.append(sc)
    # a sphere collider and a static SDF
    sc = scene.plain_grid_scene(24, 6)
    sc.options.use_sphere = True
    sc.options.sphere_center = (0.0, 0.0, -0.4)
    sc.options.sphere_radius = 0.3
    sc.static_triangles = scene.box_triangles((0.3, 0.0, -0.3), (0.2, 0.2, 0.1))
    out.append(sc)
    return out


@pytest.mark.parametrize("graphs,mode", [(True, 1), (False, 1), (True, 8)], ids=["block", "block-nographs", "cluster"])
def test_fused_batch_matches_oracle_and_launched(graphs, mode, gpu_lib, oracle_lib):
    scs = _small_mix()
    items = [(s.cloth, s.options, s.static_triangles) for s in scs]
    fused = NativeXpbdBatch(items)
    fused.set_launch_config({"fused_frame": mode})
    assert fused.launch_config()["fused_frame"] == mode
    launched = NativeXpbdBatch(items)
    launched.set_launch_config({"fused_frame": 2})
    for b in (fused, launched):
        b.set_graph_capture(graphs)
    oras = [oracle_lib.OracleSolver.from_scene(s.cloth, s.options, s.static_triangles) for s in scs]
    for frame in range(5):
        fused.step(10, 2, diagnostics=True, synchronize=True)
        launched.step(10, 2, diagnostics=True, synchronize=True)
        assert fused.last_step_launches() == 1
        assert launched.last_step_launches() > 30
        for k, o in enumerate(oras):
            o.step(10, 2)
            pf = fused.download_cloth_positions(k)
            assert np.array_equal(pf, launched.download_cloth_positions(k)), (frame, k)
            assert np.array_equal(pf, o.download_positions()), (frame, k)
        assert np.array_equal(fused.read_buffer(13, np.uint64, 38), launched.read_buffer(13, np.uint64, 38))


def test_fused_single_cloth_with_fields(gpu_lib, oracle_lib):
    """Prediction with vertex normals (volume pressure) reads the snapshot
    of other vertices: inside the fused frame those reads follow a barrier."""
    sc = scene.plain_grid_scene(20, 4)
    sc.options.use_volume_pressure = True
    sc.options.pressure_strength = 2.0
    gpu = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    assert gpu.launch_config()["fused_frame"] == 1  # one block per cloth by default
    blk = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    blk.set_launch_config({"fused_frame": 8})  # the cluster form
    ora = oracle_lib.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    for frame in range(4):
        gpu.step(10, 2, diagnostics=False, synchronize=True)
        blk.step(10, 2, diagnostics=False, synchronize=True)
        ora.step(10, 2)
        assert gpu.last_step_launches() == 1
        assert np.array_equal(gpu.download_positions(), ora.download_positions()), frame
        assert np.array_equal(blk.download_positions(), ora.download_positions()), frame


def test_large_or_self_colliding_cloths_are_not_fused(gpu_lib):
    big = scene.plain_grid_scene(40, 2)  # 1600 vertices
    s = NativeXpbdSolver(big.cloth, big.options, big.static_triangles)
    s.step(10, 2, diagnostics=False, synchronize=True)
    assert s.last_step_launches() > 1
    drop = scene.drop_scene(12, 2)
    d = NativeXpbdSolver(drop.cloth, drop.options, drop.static_triangles)
    d.step(10, 2, diagnostics=False, synchronize=True)
    assert d.last_step_launches() > 1
