"""Batched form: many cloths in one solver, each bit-identical to the oracle
run on that cloth alone.

The batch mixes cloth sizes, compliances, pin sets, fast and strict self
collision, coloured and gathered (uncoloured) bends, tethers, a static SDF
collider and a cloth without self collision.  Positions of every cloth must
equal the oracle's single-cloth run bit for bit after every frame (and so
stay inside the stated 1e-4 x extent tolerance)."""
import numpy as np
import pytest

from xpbd_gb300 import scene
from xpbd_gb300.native import NativeSolverError, NativeXpbdBatch, NativeXpbdSolver

pytestmark = pytest.mark.gpu


def _mixed_scenes():
    scs = scene.batched_scenes(5, seed=3, frames=6, side_range=(10, 26))
    # a drop scene with the static SDF collider (strict self collision)
    scs.append(scene.drop_scene(18, 6, seed=1))
    # fast self collision on the drop scene
    scs.append(scene.drop_scene(14, 6, seed=2, self_mode=1))
    # strict with a candidate budget under the 32 query slots (group queries)
    sc = scene.drop_scene(16, 6, seed=4)
    sc.options.max_self_collision_neighbors = 5
    scs.append(sc)
    # plain grid, tethers to the pins, bends gathered (no colouring)
    sc = scene.plain_grid_scene(12, 6)
    w = np.zeros(len(sc.cloth.positions_world), np.float32)
    w[sc.cloth.pin_indices] = 1.0
    sc.cloth = scene.build_cloth(sc.cloth.positions_world, sc.cloth.triangles, 0.2, w, tether_slack=1.05)
    sc.cloth.bend_color_offsets = np.asarray([0], np.int32)
    sc.options.lra_compliance = 1e-6
    scs.append(sc)
    return scs


def _oracles(scs, oracle_lib):
    return [oracle_lib.OracleSolver.from_scene(s.cloth, s.options, s.static_triangles) for s in scs]


def _items(scs):
    return [(s.cloth, s.options, s.static_triangles) for s in scs]


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_matches_each_cloth_alone(graphs, gpu_lib, oracle_lib):
    scs = _mixed_scenes()
    batch = NativeXpbdBatch(_items(scs))
    batch.set_graph_capture(graphs)
    oras = _oracles(scs, oracle_lib)
    for frame in range(5):
        batch.step(10, 2, diagnostics=False, synchronize=True)
        for k, ora in enumerate(oras):
            ora.step(10, 2)
            pg, po = batch.download_cloth_positions(k), ora.download_positions()
            err = float(np.abs(pg - po).max())
            assert err <= 1e-4 * scs[k].extent, (frame, k, err)
            assert np.array_equal(pg, po), (frame, k, err)
    # the ABI41 download on a batch handle concatenates the cloths
    allpos = batch.download_positions()
    for k, part in enumerate(batch.split_positions(allpos)):
        assert np.array_equal(part, batch.download_cloth_positions(k))


def test_batch_counters_sum_over_cloths(gpu_lib):
    """Diagnostics of a batch are the sums of its cloths' diagnostics."""
    scs = _mixed_scenes()[:4]
    batch = NativeXpbdBatch(_items(scs))
    alone = [NativeXpbdSolver(s.cloth, s.options, s.static_triangles) for s in scs]
    batch.step(10, 2, diagnostics=True)
    d = batch.diagnostics()
    keys = ("abi41_soft_contact_count", "self_candidate_count", "static_sdf_contact_count", "abi41_bending_wing_count",
            "self_filter_seen", "self_filter_cache_hits", "self_filter_cache_misses")
    sums = dict.fromkeys(keys, 0)
    for s in alone:
        s.step(10, 2, diagnostics=True)
        da = s.diagnostics()
        for k in keys:
            sums[k] += da[k]
    for k in keys:
        assert d[k] == sums[k], (k, d[k], sums[k])


def test_inactive_cloth_is_frozen_and_others_unchanged(gpu_lib, oracle_lib):
    scs = _mixed_scenes()[:4]
    batch = NativeXpbdBatch(_items(scs))
    oras = _oracles(scs, oracle_lib)
    frozen = batch.download_cloth_positions(1).copy()
    batch.set_cloth_active(1, False)
    for _ in range(3):
        batch.step(10, 2, diagnostics=False, synchronize=True)
        for k, ora in enumerate(oras):
            if k == 1:
                continue
            ora.step(10, 2)
            assert np.array_equal(batch.download_cloth_positions(k), ora.download_positions()), k
    assert np.array_equal(batch.download_cloth_positions(1), frozen)
    # re-activated, it continues like a cloth that was never stepped
    batch.set_cloth_active(1, True)
    batch.step(10, 2, diagnostics=False, synchronize=True)
    oras[1].step(10, 2)
    assert np.array_equal(batch.download_cloth_positions(1), oras[1].download_positions())


def test_batch_per_cloth_updates(gpu_lib, oracle_lib):
    """Pins, colliders and positions set on one cloth reach that cloth only."""
    scs = _mixed_scenes()[:3]
    batch = NativeXpbdBatch(_items(scs))
    oras = _oracles(scs, oracle_lib)
    batch.step(10, 2, diagnostics=False)
    for o in oras:
        o.step(10, 2)
    # move cloth 0's pins, drop cloth 2's sphere, lift cloth 1
    c0 = scs[0].cloth
    tgt = c0.pin_targets_world + np.float32(0.05)
    batch.update_cloth_pin_targets(0, c0.pin_indices, tgt, c0.pin_weights)
    oras[0].update_pin_targets(c0.pin_indices, tgt, c0.pin_weights)
    opt = scs[2].options
    opt.use_sphere = False
    batch.update_cloth_colliders(2, opt)
    from xpbd_gb300.native import colliders_from_options

    oras[2].update_runtime_colliders(colliders_from_options(opt))
    p1 = batch.download_cloth_positions(1) + np.float32(0.01)
    batch.update_cloth_positions(1, p1)
    oras[1].update_positions(p1)
    for _ in range(3):
        batch.step(10, 2, diagnostics=False, synchronize=True)
        for k, o in enumerate(oras):
            o.step(10, 2)
            assert np.array_equal(batch.download_cloth_positions(k), o.download_positions()), k


def _hard_stretch_scenes():
    scs = [scene.hardness_grid_scene(20, 1.0, 6), scene.hardness_grid_scene(16, 0.4, 6)]
    # the hard polish with greedy edge colours (no caller colouring)
    sc = scene.hardness_grid_scene(14, 1.0, 6)
    sc.cloth.edge_color_offsets = np.asarray([0], np.int32)
    scs.append(sc)
    # a cloth without the optimisation between them (spring gather)
    scs.append(scene.plain_grid_scene(12, 6))
    # the CG solve on a self-colliding drop
    sc = scene.drop_scene(14, 6, seed=5)
    sc.options.stretch_optimization_enabled = True
    sc.options.stretch_optimization_strength = 1.0
    scs.append(sc)
    return scs


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_hard_stretch_matches_each_cloth_alone(graphs, gpu_lib, oracle_lib):
    """Cloths with the CG stretch solve (strength 0.4: solve only; 1.0: plus
    averaged polish and ratio caps, with caller and greedy colourings) next
    to a spring-gather cloth in one batch: each cloth equals the oracle run
    on it alone, bit for bit, after every frame."""
    scs = _hard_stretch_scenes()
    batch = NativeXpbdBatch(_items(scs))
    batch.set_graph_capture(graphs)
    oras = _oracles(scs, oracle_lib)
    for frame in range(4):
        batch.step(10, 2, diagnostics=frame == 3, synchronize=True)
        for k, ora in enumerate(oras):
            ora.step(10, 2)
            pg, po = batch.download_cloth_positions(k), ora.download_positions()
            err = float(np.abs(pg - po).max())
            assert err <= 1e-4 * scs[k].extent, (frame, k, err)
            assert np.array_equal(pg, po), (frame, k, err)
    d = batch.diagnostics()
    solo = [NativeXpbdSolver(s.cloth, s.options, s.static_triangles) for s in scs if s.options.stretch_optimization_enabled]
    nnz = 0
    for s in solo:
        s.step(10, 2, diagnostics=True, synchronize=True)
        nnz += s.diagnostics()["abi41_pcg_csr_nnz"]
    assert d["abi41_pcg_csr_nnz"] == nnz
    assert d["abi41_pcg_iterations"] > 0 and np.isfinite(d["abi41_pcg_final_residual"])


def test_whole_handle_transfers_use_the_callers_cloth_order(gpu_lib, oracle_lib):
    """The batch stores its cloths grouped by self-collision mode; ABI41
    calls on the batch handle (whole-handle positions and pins, indices over
    the concatenation in the caller's order) still address the caller's
    cloths, and the cloth ranges describe that order."""
    scs = _mixed_scenes()
    order = [s.options.self_collision_mode if s.options.self_collision else 0 for s in scs]
    assert order != sorted(order)  # the mix is stored in another order
    batch = NativeXpbdBatch(_items(scs))
    oras = _oracles(scs, oracle_lib)
    sizes = [len(s.cloth.positions_world) for s in scs]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    for k in range(len(scs)):
        assert batch.cloth_range(k)[:2] == (int(offs[k]), sizes[k])
    # whole-handle position upload: cloth k lifted by 1 cm x (k + 1)
    allpos = np.concatenate([s.cloth.positions_world + np.float32(0.01 * (k + 1)) for k, s in enumerate(scs)])
    batch.update_positions(allpos)
    # whole-handle pins: one pin per cloth at its local vertex 3, indices over the concatenation
    idx = (offs[:-1] + 3).astype(np.int32)
    tgt = allpos[idx] + np.float32(0.02)
    batch.update_pin_targets(idx, tgt, np.ones(len(idx), np.float32))
    for k, o in enumerate(oras):
        o.update_positions(allpos[offs[k]:offs[k + 1]])
        o.update_pin_targets(np.array([3], np.int32), tgt[k:k + 1], np.ones(1, np.float32))
    for _ in range(2):
        batch.step(10, 2, diagnostics=False, synchronize=True)
        got = batch.download_positions()
        for k, o in enumerate(oras):
            o.step(10, 2)
            assert np.array_equal(got[offs[k]:offs[k + 1]], o.download_positions()), k
            assert np.array_equal(batch.download_cloth_positions(k), o.download_positions()), k
