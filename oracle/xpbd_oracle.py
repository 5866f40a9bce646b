"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loaded by the tests, the smoke check and the benchmark's CPU-baseline leg as
the checker of the GPU library; the product never imports it.  Builds
``liboracle_xpbd.so`` with the Makefile beside this file when it is missing
or older than its sources.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle_xpbd.so")
_lib = None


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("xpbd_oracle.c", "xpbd_oracle.h")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in srcs):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(LIB)
    vp, ci, pf, pi = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)
    sig = {
        "oracle_create": (vp, [vp, vp]),
        "oracle_destroy": (None, [vp]),
        "oracle_last_error": (ctypes.c_char_p, []),
        "oracle_update_pin_targets": (ci, [vp, pi, pf, pf, ci]),
        "oracle_update_runtime_colliders": (ci, [vp, vp]),
        "oracle_update_positions": (ci, [vp, pf, ci]),
        "oracle_update_static_triangles": (ci, [vp, pf, ci]),
        "oracle_update_force_fields": (ci, [vp, vp, ci]),
        "oracle_update_dynamic_triangles": (ci, [vp, pf, ci]),
        "oracle_update_dynamic_indexed": (ci, [vp, pf, ci, pi, ci, ci]),
        "oracle_update_dynamic_particles": (ci, [vp, pf, pf, ci]),
        "oracle_scene_create": (vp, []),
        "oracle_scene_destroy": (None, [vp]),
        "oracle_scene_update": (ci, [vp, vp]),
        "oracle_scene_attach": (ci, [vp, vp, ci, ci, ci]),
        "oracle_scene_clear": (ci, [vp]),
        "oracle_scene_overflow": (ctypes.c_longlong, [vp]),
        "oracle_step": (ci, [vp, ci, ci]),
        "oracle_download_positions": (ci, [vp, pf, ci]),
        "oracle_download_state": (ci, [vp, pf, pf, pf]),
        "oracle_build_self_structures": (ci, [vp]),
        "oracle_read_buffer": (ctypes.c_longlong, [vp, ci, vp, ctypes.c_longlong]),
        "oracle_hash_info": (ci, [vp, pi]),
        "oracle_dynamic_info": (ci, [vp, pi]),
        "oracle_set_threads": (ci, [ci]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    _lib = lib
    return lib


def _fp(a):
    return ctypes.POINTER(ctypes.c_float)() if a is None or a.size == 0 else a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _ip(a):
    return ctypes.POINTER(ctypes.c_int)() if a is None or a.size == 0 else a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class OracleError(RuntimeError):
    pass


class OracleSolver:
    """CPU restatement with the NativeXpbdSolver method names."""

    def __init__(self, config, mesh, keep_alive, pins=None):
        self._lib = load()
        self._h = self._lib.oracle_create(ctypes.addressof(config), ctypes.addressof(mesh))
        if not self._h:
            raise OracleError(self._lib.oracle_last_error().decode())
        self.V = config.vertex_count
        self._keep = keep_alive
        if pins is not None and len(pins[0]) > 0:
            self.update_pin_targets(*pins)

    @classmethod
    def from_scene(cls, cloth, options, static_triangles):
        import sys

        pkg = os.path.join(os.path.dirname(HERE), "ssbl-cuda-xpbd_gb300")
        if pkg not in sys.path:
            sys.path.insert(0, pkg)
        from xpbd_gb300.native import config_from_options, mesh_arrays

        cfg = config_from_options(cloth, options, static_triangles)
        mesh, keep = mesh_arrays(cloth, static_triangles)
        return cls(cfg, mesh, keep, (cloth.pin_indices, cloth.pin_targets_world, cloth.pin_weights))

    def _check(self, ok):
        if not ok:
            raise OracleError(self._lib.oracle_last_error().decode())

    def close(self):
        if self._h:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update_pin_targets(self, indices, positions, weights=None):
        idx = np.ascontiguousarray(indices, np.int32)
        pos = np.ascontiguousarray(positions, np.float32)
        w = None if weights is None else np.ascontiguousarray(weights, np.float32)
        self._check(self._lib.oracle_update_pin_targets(self._h, _ip(idx), _fp(pos), _fp(w), len(idx)))

    def update_runtime_colliders(self, colliders):
        self._check(self._lib.oracle_update_runtime_colliders(self._h, ctypes.addressof(colliders)))

    def update_positions(self, positions):
        p = np.ascontiguousarray(positions, np.float32)
        self._check(self._lib.oracle_update_positions(self._h, _fp(p), p.size))

    def update_static_triangles(self, tris):
        t = np.ascontiguousarray(np.asarray(tris, np.float32).reshape(-1, 3))
        self._check(self._lib.oracle_update_static_triangles(self._h, _fp(t), len(t) // 3))

    def update_force_fields(self, fields):
        """`fields`: a ctypes array of NativeForceField records."""
        n = len(fields)
        self._check(self._lib.oracle_update_force_fields(self._h, ctypes.addressof(fields) if n else None, n))

    def update_dynamic_colliders(self, *, triangles=None, indexed=None, particles=None):
        """Same arguments as NativeXpbdSolver.update_dynamic_colliders."""
        if triangles is not None:
            t = np.ascontiguousarray(np.asarray(triangles, np.float32).reshape(-1, 9))
            self._check(self._lib.oracle_update_dynamic_triangles(self._h, _fp(t), len(t)))
        if indexed is not None:
            verts, idx, changed = indexed
            v = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, 3))
            ix = np.ascontiguousarray(np.asarray(idx, np.int32).reshape(-1, 3))
            self._check(self._lib.oracle_update_dynamic_indexed(self._h, _fp(v), len(v), _ip(ix), len(ix), 1 if changed else 0))
        if particles is not None:
            pos, rad = particles
            p = np.ascontiguousarray(np.asarray(pos, np.float32).reshape(-1, 3))
            r = np.ascontiguousarray(np.asarray(rad, np.float32).reshape(-1))
            self._check(self._lib.oracle_update_dynamic_particles(self._h, _fp(p), _fp(r), len(p)))

    def attach_global_scene(self, scene, target_source_id=0, target_collision_layer=0, mode=1):
        self._check(self._lib.oracle_scene_attach(self._h, scene._h, int(target_source_id), int(target_collision_layer), int(mode)))
        self._scene_ref = scene

    def clear_global_scene(self):
        self._check(self._lib.oracle_scene_clear(self._h))
        self._scene_ref = None

    def step(self, substeps, iterations):
        self._check(self._lib.oracle_step(self._h, int(substeps), int(iterations)))

    def download_positions(self):
        out = np.empty((self.V, 3), np.float32)
        self._check(self._lib.oracle_download_positions(self._h, _fp(out), out.size))
        return out

    def download_state(self):
        p, q, v = (np.empty((self.V, 3), np.float32) for _ in range(3))
        self._check(self._lib.oracle_download_state(self._h, _fp(p), _fp(q), _fp(v)))
        return p, q, v

    def build_self_structures(self):
        self._check(self._lib.oracle_build_self_structures(self._h))

    def read_buffer(self, which, dtype, count):
        out = np.empty(count, dtype=dtype)
        n = self._lib.oracle_read_buffer(self._h, int(which), out.ctypes.data, out.nbytes)
        if n < 0:
            raise OracleError(self._lib.oracle_last_error().decode())
        return out[: n // out.itemsize]

    def hash_info(self):
        out = np.zeros(6, np.int32)
        self._check(self._lib.oracle_hash_info(self._h, _ip(out)))
        return out


    def dynamic_info(self):
        out = np.zeros(6, np.int32)
        self._check(self._lib.oracle_dynamic_info(self._h, _ip(out)))
        return {"triangles": int(out[0]), "large": int(out[1]), "max_occupancy": int(out[2]), "tri_hashed": bool(out[3]),
                "particles": int(out[4]), "par_hashed": bool(out[5])}


class OracleScene:
    """Shared dynamic scene of the oracle (same arguments as
    xpbd_gb300.native.GlobalDynamicScene)."""

    def __init__(self):
        self._lib = load()
        self._h = self._lib.oracle_scene_create()

    def update(self, triangles=None, particles=None, margin: float = 0.0, thickness: float = 0.0):
        import sys

        pkg = os.path.join(os.path.dirname(HERE), "ssbl-cuda-xpbd_gb300")
        if pkg not in sys.path:
            sys.path.insert(0, pkg)
        from xpbd_gb300.native import scene_inputs

        fi, keep = scene_inputs(triangles, particles, margin, thickness)
        if not self._lib.oracle_scene_update(self._h, ctypes.addressof(fi)):
            raise OracleError(self._lib.oracle_last_error().decode())
        del keep

    def overflow(self) -> int:
        return int(self._lib.oracle_scene_overflow(self._h))

    def close(self):
        if self._h:
            self._lib.oracle_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_threads(n: int) -> int:
    return int(load().oracle_set_threads(int(n)))
