"""PC2 point caches: the streaming writer of the library (device transform,
pinned double buffer, writer thread) and a reader for the format of the
reference add-on's bake (session_manager.py:4624-4643): a 32-byte header
'<12siiffi' (b"POINTCACHE2\\0", version 1, vertex count, start frame,
sample rate 1.0, sample count) followed by float32 xyz per vertex per
sample, in object-local coordinates."""
from __future__ import annotations

import ctypes
import struct

import numpy as np

from .native import NativeSolverError, _last_error, _load_library

HEADER = struct.Struct("<12siiffi")


def _lib():
    lib = _load_library()
    if not getattr(lib, "_pc2_bound", False):
        vp = ctypes.c_void_p
        lib.xpbd_gb300_pc2_open.argtypes = [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
        lib.xpbd_gb300_pc2_open.restype = vp
        lib.xpbd_gb300_pc2_write.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_float)]
        lib.xpbd_gb300_pc2_write.restype = ctypes.c_int
        lib.xpbd_gb300_pc2_close.argtypes = [vp, ctypes.c_int]
        lib.xpbd_gb300_pc2_close.restype = ctypes.c_longlong
        lib._pc2_bound = True
    return lib


class Pc2Writer:
    """Streams one cloth of a solver (or batch cloth index) to a PC2 file."""

    def __init__(self, solver, path: str, start_frame: int, cloth: int = -1):
        self._lib = _lib()
        self._solver = solver
        self._w = self._lib.xpbd_gb300_pc2_open(solver.handle, int(cloth), str(path).encode(), int(start_frame))
        if not self._w:
            raise NativeSolverError(_last_error(self._lib))

    def write(self, matrix_world_inv=None) -> None:
        """Append the cloth's current positions (object-local through the
        inverse object matrix, 4x4; None = world)."""
        m = None
        if matrix_world_inv is not None:
            m = np.ascontiguousarray(np.asarray(matrix_world_inv, np.float32).reshape(4, 4))
        ptr = m.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if m is not None else None
        if not self._lib.xpbd_gb300_pc2_write(self._solver.handle, self._w, ptr):
            raise NativeSolverError(_last_error(self._lib))

    def close(self, commit: bool = True) -> int:
        if not self._w:
            return 0
        n = self._lib.xpbd_gb300_pc2_close(self._w, 1 if commit else 0)
        self._w = None
        if n < 0:
            raise NativeSolverError(_last_error(self._lib))
        return int(n)

    def __del__(self):
        try:
            if self._w:
                self.close(commit=False)
        except Exception:
            pass


def read_pc2(path: str):
    """(header dict, samples (S, V, 3) float32)."""
    with open(path, "rb") as f:
        raw = f.read()
    magic, version, count, start, rate, samples = HEADER.unpack_from(raw, 0)
    data = np.frombuffer(raw, dtype="<f4", offset=HEADER.size)
    return ({"magic": magic, "version": version, "vertex_count": count, "start_frame": start, "sample_rate": rate,
             "samples": samples}, data.reshape(samples, count, 3) if samples else data.reshape(0, count, 3))


def to_local(world: np.ndarray, matrix_inv: np.ndarray) -> np.ndarray:
    """The reference's object-local transform in float32
    (xpbd_core.py:652-655)."""
    world = np.asarray(world, dtype=np.float32)
    matrix_inv = np.asarray(matrix_inv, dtype=np.float32)
    return world @ matrix_inv[:3, :3].T + matrix_inv[:3, 3]
