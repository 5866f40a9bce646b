"""The allocation-free vertex hash entry point against the solver's own hash.

Callers such as host applications that reserve all device memory through
their own pool, or frame loops that cannot afford the device synchronisation
of cudaMalloc / cudaFree, use xpbd_gb300_vertex_hash_noalloc: it takes device
inputs and outputs and keeps its only scratch (bucket counters) in a
fixed-size array inside the library.  This test calls it through the C-ABI
twice in a row, on two different cloth configurations, and requires the same
integers as the solver's existing hash build (xpbd_gb300_build_self_structures)
on the same positions: cells, bucket ranges, and bucket members.  The file is
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _folded(sc, seed, offset):
    rng = np.random.default_rng(seed)
    p = sc.cloth.positions_world.copy()
    right = p[:, 0] > 0.0
    p[right, 0] = -p[right, 0] + offset
    p[right, 2] += 0.0012
    p[:, :2] += rng.uniform(-2e-4, 2e-4, (len(p), 2)).astype(np.float32)
    return np.ascontiguousarray(p, np.float32)


def test_vertex_hash_noalloc_matches_solver_hash(gpu_lib):
    import torch

    from xpbd_gb300 import native, scene

    lib = native._load_library()
    fn = lib.xpbd_gb300_vertex_hash_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    sc = scene.drop_scene(64, 1, seed=5)
    solver = native.NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    V = len(sc.cloth.positions_world)
    nvb = int(solver.hash_info()[0])
    radius = np.float32(max(sc.options.cloth_thickness, sc.options.collision_margin))
    cell = float(max(np.float32(radius * np.float32(1.8)), np.float32(1e-3)))
    dev = torch.device("cuda:0")
    for call, (seed, offset) in enumerate(((11, 0.001), (12, 0.0015))):
        p = _folded(sc, seed, offset)
        solver.update_positions(p)
        solver.build_self_structures()
        ref_cells = solver.read_buffer(3, np.int32, 4 * V)
        ref_start = solver.read_buffer(4, np.int32, nvb + 1)
        ref_ent = solver.read_buffer(5, np.int32, V)
        d_pos = torch.from_numpy(p).to(dev)
        d_start = torch.full((nvb + 1,), -7, dtype=torch.int32, device=dev)
        d_ent = torch.full((V,), -7, dtype=torch.int32, device=dev)
        d_cells = torch.full((4 * V,), -7, dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        ok = fn(d_pos.data_ptr(), V, cell, nvb, d_start.data_ptr(), d_ent.data_ptr(), d_cells.data_ptr(), stream)
        assert ok == 1, native._last_error(lib)
        torch.cuda.synchronize()
        start, ent, cells = d_start.cpu().numpy(), d_ent.cpu().numpy(), d_cells.cpu().numpy()
        assert np.array_equal(cells, ref_cells), call
        assert np.array_equal(start, ref_start), call
        for b in np.flatnonzero(np.diff(start)):
            lo, hi = start[b], start[b + 1]
            assert np.array_equal(np.sort(ent[lo:hi]), np.sort(ref_ent[lo:hi])), (call, b)
            n = min(hi - lo, 32)
            assert np.array_equal(ent[lo:lo + n], ref_ent[lo:lo + n]), (call, b)
    # sizes beyond the fixed scratch are refused with a clear error
    d_start = torch.zeros((1 << 19) + 1, dtype=torch.int32, device=dev)
    assert fn(d_pos.data_ptr(), V, cell, 1 << 19, d_start.data_ptr(), d_ent.data_ptr(), 0, 0) == 0
    assert b"262144" in lib.ssbl_last_error()
    solver.close()
