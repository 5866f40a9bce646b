"""The C-ABI library builds, loads without a GPU and exports every entry
point the public headers declare."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in ("ssbl_xpbd_cuda.h", "xpbd_gb300.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        names += re.findall(r"\b((?:ssbl|xpbd_gb300)_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from xpbd_gb300 import build

    return ctypes.CDLL(build.build())


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 26
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi41_core_set_present(lib):
    core = """ssbl_create_solver ssbl_destroy_solver ssbl_reset_solver ssbl_update_pin_targets
    ssbl_update_runtime_colliders ssbl_update_positions ssbl_update_static_triangles ssbl_update_dynamic_triangles
    ssbl_update_frame_inputs ssbl_step_solver ssbl_step_solver_ex ssbl_download_positions ssbl_get_diagnostics
    ssbl_capabilities ssbl_create_global_dynamic_scene ssbl_destroy_global_dynamic_scene
    ssbl_update_global_dynamic_scene ssbl_attach_global_dynamic_scene ssbl_clear_global_dynamic_scene
    ssbl_last_error""".split()
    assert len(core) == 20
    for n in core:
        assert hasattr(lib, n), n


def test_capabilities_without_gpu(lib):
    lib.ssbl_capabilities.restype = ctypes.c_uint
    assert lib.ssbl_capabilities() == 7


def test_error_convention_without_gpu(lib):
    """Invalid handles fail with 0 and a message, like the reference."""
    lib.ssbl_step_solver_ex.restype = ctypes.c_int
    lib.ssbl_last_error.restype = ctypes.c_char_p
    assert lib.ssbl_step_solver_ex(None, 1, 1, 0, 0) == 0
    assert lib.ssbl_last_error() == b"invalid solver handle"
    lib.ssbl_create_solver.restype = ctypes.c_void_p
    assert not lib.ssbl_create_solver(None, None)
    assert lib.ssbl_last_error() == b"invalid ABI41 solver create request"
