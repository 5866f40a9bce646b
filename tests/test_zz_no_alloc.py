"""The allocation-free vertex hash entry point against the solver's own hash.

Some callers cannot call cudaMalloc / cudaFree: host applications that
reserve all device memory up front through their own pool, and frame loops
that cannot afford the device synchronisation those calls may bring.  They
use xpbd_gb300_vertex_hash_noalloc, which takes device inputs and outputs and
keeps its only scratch (bucket counters) in a fixed-size array inside the
library.  This test calls it through the C-ABI twice in a row, on two fold
offsets of the same 64x64 cloth, and requires the same integers as the
solver's existing hash build (xpbd_gb300_build_self_structures) on the same
positions: cells, bucket ranges and bucket members.  It also covers a crowded
bucket (every vertex in one cell, ordered by a warp), the largest accepted
table (262,144 buckets, checked against the same hash computed on the host),
an empty vertex set, a NULL cells pointer and the refusal of a larger table.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 18


def _folded(sc, seed, offset):
    rng = np.random.default_rng(seed)
    p = sc.cloth.positions_world.copy()
    right = p[:, 0] > 0.0
    p[right, 0] = -p[right, 0] + offset
    p[right, 2] += 0.0012
    p[:, :2] += rng.uniform(-2e-4, 2e-4, (len(p), 2)).astype(np.float32)
    return np.ascontiguousarray(p, np.float32)


def _entry(lib):
    fn = lib.xpbd_gb300_vertex_hash_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    return fn


def _check_against(start, ent, ref_start, ref_ent, tag):
    assert np.array_equal(start, ref_start), tag
    for b in np.flatnonzero(np.diff(start)):
        lo, hi = start[b], start[b + 1]
        assert np.array_equal(np.sort(ent[lo:hi]), np.sort(ref_ent[lo:hi])), (tag, b)
        n = min(hi - lo, 32)
        assert np.array_equal(ent[lo:lo + n], ref_ent[lo:lo + n]), (tag, b)


def test_vertex_hash_noalloc_matches_solver_hash(gpu_lib):
    import torch

    from xpbd_gb300 import native, scene

    lib = native._load_library()
    fn = _entry(lib)
    sc = scene.drop_scene(64, 1, seed=5)
    solver = native.NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    V = len(sc.cloth.positions_world)
    nvb = int(solver.hash_info()[0])
    radius = np.float32(max(sc.options.cloth_thickness, sc.options.collision_margin))
    cell = float(max(np.float32(radius * np.float32(1.8)), np.float32(1e-3)))
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(3)
    collapsed = np.full((V, 3), 0.0007, np.float32) + rng.uniform(0, 1e-4, (V, 3)).astype(np.float32)
    cases = [("call 1", _folded(sc, 11, 0.001)), ("call 2", _folded(sc, 12, 0.0015)), ("crowded", collapsed)]
    for tag, p in cases:
        solver.update_positions(p)
        solver.build_self_structures()
        ref_cells = solver.read_buffer(3, np.int32, 4 * V)
        ref_start = solver.read_buffer(4, np.int32, nvb + 1)
        ref_ent = solver.read_buffer(5, np.int32, V)
        d_pos = torch.from_numpy(p).to(dev)
        d_start = torch.full((nvb + 1,), -7, dtype=torch.int32, device=dev)
        d_ent = torch.full((V,), -7, dtype=torch.int32, device=dev)
        d_cells = torch.full((4 * V,), -7, dtype=torch.int32, device=dev)
        ok = fn(d_pos.data_ptr(), V, cell, nvb, d_start.data_ptr(), d_ent.data_ptr(), d_cells.data_ptr(), stream)
        assert ok == 1, native._last_error(lib)
        torch.cuda.synchronize()
        start, ent, cells = d_start.cpu().numpy(), d_ent.cpu().numpy(), d_cells.cpu().numpy()
        assert np.array_equal(cells, ref_cells), tag
        _check_against(start, ent, ref_start, ref_ent, tag)
        if tag == "crowded":
            assert np.diff(start).max() > 32  # the warp-ordered path ran

    # the largest accepted table, no cells output: the same hash on the host
    p = cases[0][1]
    solver.update_positions(p)
    solver.build_self_structures()
    c = solver.read_buffer(3, np.int32, 4 * V).reshape(V, 4)[:, :3].astype(np.int64) & 0xFFFFFFFF
    h = ((c[:, 0] * 73856093) ^ (c[:, 1] * 19349663) ^ (c[:, 2] * 83492791)) & (LIMIT - 1)
    counts = np.bincount(h, minlength=LIMIT)
    want_start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    d_pos = torch.from_numpy(p).to(dev)
    d_start = torch.full((LIMIT + 1,), -7, dtype=torch.int32, device=dev)
    d_ent = torch.full((V,), -7, dtype=torch.int32, device=dev)
    assert fn(d_pos.data_ptr(), V, cell, LIMIT, d_start.data_ptr(), d_ent.data_ptr(), None, stream) == 1
    torch.cuda.synchronize()
    start, ent = d_start.cpu().numpy(), d_ent.cpu().numpy()
    assert np.array_equal(start, want_start)
    order = np.argsort(h, kind="stable")  # ids ascending within each bucket
    assert np.array_equal(ent, order.astype(np.int32))

    # no vertices: every bucket empty
    d_start.fill_(-7)
    assert fn(d_pos.data_ptr(), 0, cell, nvb, d_start.data_ptr(), d_ent.data_ptr(), None, stream) == 1
    torch.cuda.synchronize()
    assert not d_start[: nvb + 1].cpu().numpy().any()

    # sizes beyond the fixed scratch are refused with a clear error
    d_start = torch.zeros((1 << 19) + 1, dtype=torch.int32, device=dev)
    assert fn(d_pos.data_ptr(), V, cell, 1 << 19, d_start.data_ptr(), d_ent.data_ptr(), None, None) == 0
    assert b"262144" in lib.ssbl_last_error()
    solver.close()
