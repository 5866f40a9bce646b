"""GB300-native XPBD cloth solver: the ABI41 drop-in library and its host side.

* ``build``  -- nvcc recipe of ``lib/libssbl_xpbd_cuda_abi41.so`` (sm_103a)
* ``native`` -- ctypes mirror of the reference bridge (``NativeXpbdSolver``)
* ``scene``  -- synthetic cloths and the constraint builders of the reference
"""
from .native import NativeBackendUnavailable, NativeSolverError, NativeXpbdSolver  # noqa: F401
from .scene import ClothData, SolverOptions  # noqa: F401

__all__ = ["NativeXpbdSolver", "NativeSolverError", "NativeBackendUnavailable", "ClothData", "SolverOptions"]
