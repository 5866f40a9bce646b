"""The reference's own CUDA solver, driven from Python (test infrastructure).

Loads oracle/_ref/libssbl_xpbd_cuda_abi41_ref.so (built by oracle/build_ref.py
from the reference's sources, with the probe of oracle/ref_probe.cu in the
same translation unit) through the same ctypes mirror of the ABI41 structs
that drives this repository's library, so both solvers receive byte-identical
configs, meshes and pins.  Used only by the parity tests and by the
benchmark's reference timings; the product never loads it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libssbl_xpbd_cuda_abi41_ref.so")
SMOKE_REF = os.path.join(HERE, "_ref", "abi41_smoke_ref")
SMOKE_PRODUCT = os.path.join(HERE, "_ref", "abi41_smoke_product")

# Buffer ids of refprobe_read (oracle/ref_probe.cu).
VERTEX_CELLS, VERTEX_BUCKET_COUNTS, VERTEX_BUCKET_SLOTS = 0, 1, 2
TRI_CELLS, TRI_BUCKET_COUNTS, TRI_BUCKET_SLOTS = 3, 4, 5
EDGE_CELLS, EDGE_BUCKET_COUNTS, EDGE_BUCKET_SLOTS = 6, 7, 8
NEIGHBOR_COUNTS, NEIGHBOR_SLOTS, COUNTERS = 9, 10, 11
POSITIONS, PREVIOUS, VELOCITIES = 12, 13, 14
SLOTS = 32


def available() -> bool:
    return os.path.exists(REF_LIB)


def _probe_lib():
    from xpbd_gb300 import native

    lib = native._load_library(REF_LIB)
    vp = ctypes.c_void_p
    lib.refprobe_hash_info.restype = ctypes.c_int
    lib.refprobe_hash_info.argtypes = [vp, vp, vp]
    lib.refprobe_set_state.restype = ctypes.c_int
    lib.refprobe_set_state.argtypes = [vp, vp, vp]
    lib.refprobe_build_self_structures.restype = ctypes.c_int
    lib.refprobe_build_self_structures.argtypes = [vp]
    lib.refprobe_read.restype = ctypes.c_longlong
    lib.refprobe_read.argtypes = [vp, ctypes.c_int, vp, ctypes.c_longlong]
    lib.refprobe_cell_coords.restype = ctypes.c_int
    lib.refprobe_cell_coords.argtypes = [vp, ctypes.c_int, ctypes.c_float, vp]
    return lib


class RefSolver:
    """One reference solver (the unchanged ABI41 entry points plus the probe)."""

    def __init__(self, cloth, options, static_triangles):
        from xpbd_gb300 import native

        self._lib = _probe_lib()
        self.solver = native.NativeXpbdSolver(cloth, options, static_triangles, library=REF_LIB)
        self.V = len(cloth.positions_world)

    @classmethod
    def from_scene(cls, sc):
        return cls(sc.cloth, sc.options, sc.static_triangles)

    @property
    def handle(self):
        return self.solver.handle

    def step(self, substeps, iterations, diagnostics=True, synchronize=True):
        self.solver.step(substeps, iterations, diagnostics=diagnostics, synchronize=synchronize)

    def download_positions(self) -> np.ndarray:
        return self.solver.download_positions().copy()

    def diagnostics(self) -> dict:
        return self.solver.diagnostics()

    def close(self):
        self.solver.close()

    def hash_info(self):
        out = np.zeros(8, np.int32)
        cells = np.zeros(3, np.float32)
        if not self._lib.refprobe_hash_info(self.handle, out.ctypes.data, cells.ctypes.data):
            raise RuntimeError("refprobe_hash_info failed")
        return out, cells

    def set_state(self, pos: np.ndarray, prev: np.ndarray | None = None):
        pos = np.ascontiguousarray(pos, np.float32)
        prev = None if prev is None else np.ascontiguousarray(prev, np.float32)
        ok = self._lib.refprobe_set_state(self.handle, pos.ctypes.data, None if prev is None else prev.ctypes.data)
        if not ok:
            raise RuntimeError("refprobe_set_state failed")

    def build_self_structures(self):
        if not self._lib.refprobe_build_self_structures(self.handle):
            raise RuntimeError("refprobe_build_self_structures failed")

    def read(self, which: int, dtype, count: int) -> np.ndarray:
        out = np.zeros(max(int(count), 1), dtype)
        n = self._lib.refprobe_read(self.handle, which, out.ctypes.data, out.nbytes)
        if n < 0:
            raise RuntimeError(f"refprobe_read({which}) failed")
        return out[: n // out.itemsize]

    def state(self):
        V = self.V
        return (self.read(POSITIONS, np.float32, 3 * V).reshape(V, 3),
                self.read(PREVIOUS, np.float32, 3 * V).reshape(V, 3),
                self.read(VELOCITIES, np.float32, 3 * V).reshape(V, 3))


def cell_coords(values: np.ndarray, cell: float) -> np.ndarray:
    """The reference's cell_coord on the GPU, for each value."""
    lib = _probe_lib()
    v = np.ascontiguousarray(values, np.float32)
    out = np.zeros(len(v), np.int32)
    if not lib.refprobe_cell_coords(v.ctypes.data, len(v), float(cell), out.ctypes.data):
        raise RuntimeError("refprobe_cell_coords failed")
    return out
