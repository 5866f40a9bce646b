"""GPU library against the reference's known-answer smoke cases, and against
the oracle on the same cases (bit-identical positions expected; the stated
tolerance is 1e-4 of the case extent)."""
import numpy as np
import pytest

import kat_cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make", kat_cases.ALL, ids=lambda f: f.__name__)
def test_gpu_known_answers_and_oracle_parity(make, gpu_lib, oracle_lib):
    case, run = make()
    gpu = gpu_lib.NativeXpbdSolver.from_raw(case.cfg, case.mesh, case.pins)
    out_gpu = run(gpu)
    case2, run2 = make()
    ora = oracle_lib.OracleSolver(case2.cfg, case2.mesh, case2.keep, case2.pins)
    out_ora = run2(ora)
    extent = max(float(np.ptp(out_ora, axis=0).max()), 1e-3)
    err = float(np.abs(out_gpu - out_ora).max())
    assert err <= 1e-4 * extent, err
    assert np.array_equal(out_gpu, out_ora), f"not bit-identical, max err {err}"
    gpu.close()


def test_gpu_self_diagnostics(gpu_lib):
    """abi41_smoke.cpp:292-306: contacts, candidates and the smoothed delta
    are reported in the diagnostics block."""
    case, run = kat_cases.self_vv()
    gpu = gpu_lib.NativeXpbdSolver.from_raw(case.cfg, case.mesh, case.pins)
    run(gpu)
    d = gpu.diagnostics()
    assert d["finite_flag"] == 1
    assert d["abi41_soft_contact_count"] + d["abi41_exact_impulse_contact_count"] > 0
    assert d["fast_soft_repulsion_candidates"] > 0
    assert d["abi41_max_smoothed_delta"] > 0.0


def test_gpu_sdf_diagnostics_and_rebuild(gpu_lib):
    """abi41_smoke.cpp:115-127, 170-220: SDF grid, contact and rebuild counts."""
    case, run = kat_cases.static_sdf_plane()
    gpu = gpu_lib.NativeXpbdSolver.from_raw(case.cfg, case.mesh, case.pins)
    run(gpu)
    d = gpu.diagnostics()
    assert d["static_sdf_rebuild_count"] > 0 and d["static_sdf_voxel_count"] > 0
    assert min(d["static_sdf_grid_x"], d["static_sdf_grid_y"], d["static_sdf_grid_z"]) > 1
    assert d["static_sdf_contact_count"] > 0 and d["static_sdf_unsigned_fallback_count"] > 0
    r0 = d["static_sdf_rebuild_count"]
    gpu.update_static_triangles(kat_cases.box_triangles(0.5))
    gpu.step(1, 2)
    d2 = gpu.diagnostics()
    assert d2["static_sdf_rebuild_count"] > r0 and d2["static_triangle_count"] == 12
    small = np.array([[-0.6, -0.6, 0.2], [0.6, -0.6, 0.2], [-0.6, 0.6, 0.2], [0.6, -0.6, 0.2], [0.6, 0.6, 0.2],
                      [-0.6, 0.6, 0.2]], np.float32).reshape(2, 3, 3)
    gpu.update_static_triangles(small)
    d3 = gpu.diagnostics()
    assert d3["static_sdf_rebuild_count"] > d2["static_sdf_rebuild_count"] and d3["static_triangle_count"] == 2


def test_gpu_bend_wing_diagnostics(gpu_lib):
    """abi41_smoke.cpp:1063-1077: wings reported, texture flag set."""
    case, run = kat_cases.bend_hinge()
    gpu = gpu_lib.NativeXpbdSolver.from_raw(case.cfg, case.mesh, case.pins)
    run(gpu)
    d = gpu.diagnostics()
    assert d["abi41_bending_texture_ready"] == 1 and d["abi41_bending_wing_count"] > 0


def test_gpu_hard_stretch_known_answers_and_parity(gpu_lib, oracle_lib):
    """abi41_smoke.cpp:599-876: PCG shrinks a stretched edge more than the
    soft springs, keeps pins, CSR nnz 2 / 6, residual decreases; outputs
    bit-identical to the oracle."""
    diags = {}

    def make_gpu(c):
        s = gpu_lib.NativeXpbdSolver.from_raw(c.cfg, c.mesh, c.pins)
        diags[len(diags)] = s
        return s

    g = kat_cases.hard_stretch_suite(make_gpu)
    o = kat_cases.hard_stretch_suite(lambda c: oracle_lib.OracleSolver(c.cfg, c.mesh, c.keep, c.pins))
    for k in g:
        assert np.array_equal(g[k], o[k]), (k, g[k], o[k])
    on = diags[1].diagnostics()
    assert on["abi41_pcg_csr_nnz"] == 2 and on["abi41_pcg_texture_ready"] == 1 and on["abi41_pcg_iterations"] > 0
    assert on["abi41_pcg_initial_residual"] > 0.0
    assert on["abi41_pcg_final_residual"] < on["abi41_pcg_initial_residual"]
    assert on["abi41_pcg_max_delta"] > 0.0
    chain = diags[5].diagnostics()
    assert chain["abi41_pcg_csr_nnz"] == 6 and chain["abi41_pcg_iterations"] > 0
    assert chain["abi41_pcg_final_residual"] < chain["abi41_pcg_initial_residual"]
