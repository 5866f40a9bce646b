"""Differentiable form: per-constraint compliances -> final cloth positions,
with the library's hand-written adjoint behind a torch.autograd.Function.

The rollout is the contact-free XPBD step of the solver (stretch and bend
constraints, hard pins, the velocity update) run on the GPU from the rest
state for `frames` frames; every frame's starting state is kept as a
checkpoint and the backward pass recomputes one frame at a time from its
checkpoint before propagating the adjoint through it.  PyTorch only carries
the tensors (device pointers go straight to the C entry points).
"""
from __future__ import annotations

import ctypes

import numpy as np

from .native import NativeSolverError, _fp, _ip, _last_error, _load_library, config_from_options, mesh_arrays
from .scene import ClothData, SolverOptions

_VP = ctypes.c_void_p


def _lib():
    lib = _load_library()
    if not getattr(lib, "_diff_bound", False):
        pf = ctypes.POINTER(ctypes.c_float)
        pi = ctypes.POINTER(ctypes.c_int)
        from .native import NativeConfig, NativeMesh

        lib.xpbd_gb300_diff_create.argtypes = [ctypes.POINTER(NativeConfig), ctypes.POINTER(NativeMesh)]
        lib.xpbd_gb300_diff_create.restype = _VP
        lib.xpbd_gb300_diff_destroy.argtypes = [_VP]
        lib.xpbd_gb300_diff_destroy.restype = ctypes.c_int
        lib.xpbd_gb300_diff_update_pin_targets.argtypes = [_VP, pi, pf, pf, ctypes.c_int]
        lib.xpbd_gb300_diff_update_pin_targets.restype = ctypes.c_int
        lib.xpbd_gb300_diff_rollout.argtypes = [_VP, _VP, _VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP]
        lib.xpbd_gb300_diff_rollout.restype = ctypes.c_int
        lib.xpbd_gb300_diff_backward.argtypes = [_VP, _VP, _VP, _VP]
        lib.xpbd_gb300_diff_backward.restype = ctypes.c_int
        lib.xpbd_gb300_diff_checkpoint.argtypes = [_VP, ctypes.c_int, _VP]
        lib.xpbd_gb300_diff_checkpoint.restype = ctypes.c_int
        lib._diff_bound = True
    return lib


class DiffCloth:
    """A contact-free cloth for differentiable rollouts (one GPU handle)."""

    def __init__(self, cloth: ClothData, options: SolverOptions):
        self._lib = _lib()
        cfg = config_from_options(cloth, options, np.empty((0, 3, 3), np.float32))
        mesh, keep = mesh_arrays(cloth, np.empty((0, 3, 3), np.float32))
        self._handle = self._lib.xpbd_gb300_diff_create(ctypes.byref(cfg), ctypes.byref(mesh))
        del keep
        if not self._handle:
            raise NativeSolverError(_last_error(self._lib))
        self.vertex_count = len(cloth.positions_world)
        self.edge_count = len(cloth.edges)
        self.bend_count = len(cloth.bends)
        self.rollout_id = 0
        if len(cloth.pin_indices) > 0:
            idx = np.ascontiguousarray(cloth.pin_indices, np.int32)
            pos = np.ascontiguousarray(cloth.pin_targets_world, np.float32)
            w = np.ascontiguousarray(cloth.pin_weights, np.float32)
            if not self._lib.xpbd_gb300_diff_update_pin_targets(self._handle, _ip(idx), _fp(pos), _fp(w), len(idx)):
                raise NativeSolverError(_last_error(self._lib))

    def close(self):
        if getattr(self, "_handle", None):
            self._lib.xpbd_gb300_diff_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rollout(self, stretch, bend, frames: int, substeps: int = 10, iterations: int = 2):
        """Final positions (V, 3) for per-edge / per-bend compliances (CUDA
        float32 tensors of E and B values)."""
        import torch

        stretch = stretch.detach().contiguous().float()
        bend = bend.detach().contiguous().float()
        out = torch.empty((self.vertex_count, 3), dtype=torch.float32, device=stretch.device)
        torch.cuda.current_stream().synchronize()
        ok = self._lib.xpbd_gb300_diff_rollout(self._handle, stretch.data_ptr() if stretch.numel() else None,
                                               bend.data_ptr() if bend.numel() else None, int(frames), int(substeps),
                                               int(iterations), out.data_ptr())
        if not ok:
            raise NativeSolverError(_last_error(self._lib))
        self.rollout_id += 1
        return out

    def backward(self, grad_positions):
        """dL/d(stretch compliance), dL/d(bend compliance) of the last rollout
        for dL/d(final positions) = grad_positions."""
        import torch

        g = grad_positions.detach().contiguous().float()
        gs = torch.empty(self.edge_count, dtype=torch.float32, device=g.device)
        gb = torch.empty(self.bend_count, dtype=torch.float32, device=g.device)
        torch.cuda.current_stream().synchronize()
        ok = self._lib.xpbd_gb300_diff_backward(self._handle, g.data_ptr(), gs.data_ptr() if gs.numel() else None,
                                                gb.data_ptr() if gb.numel() else None)
        if not ok:
            raise NativeSolverError(_last_error(self._lib))
        return gs, gb

    def checkpoint(self, frame: int):
        """State at the start of `frame` of the last rollout (frame = frames:
        the final state): a (3, V, 4) CUDA tensor of positions, previous
        positions and velocities (xyz + a fourth lane)."""
        import torch

        out = torch.empty((3, self.vertex_count, 4), dtype=torch.float32, device="cuda")
        torch.cuda.current_stream().synchronize()
        if not self._lib.xpbd_gb300_diff_checkpoint(self._handle, int(frame), out.data_ptr()):
            raise NativeSolverError(_last_error(self._lib))
        return out


def _autograd_function():
    import torch

    class XpbdRollout(torch.autograd.Function):
        """positions = rollout(stretch compliance per edge, bend compliance per
        bend); backward by the library's adjoint with per-frame
        checkpointing."""

        @staticmethod
        def forward(ctx, stretch, bend, cloth: DiffCloth, frames: int, substeps: int, iterations: int):
            out = cloth.rollout(stretch, bend, frames, substeps, iterations)
            ctx.cloth = cloth
            ctx.args = (frames, substeps, iterations)
            ctx.rollout_id = cloth.rollout_id
            ctx.save_for_backward(stretch, bend)
            return out

        @staticmethod
        def backward(ctx, grad_out):
            stretch, bend = ctx.saved_tensors
            cloth = ctx.cloth
            if cloth.rollout_id != ctx.rollout_id:  # another rollout ran since: recompute this one's checkpoints
                cloth.rollout(stretch, bend, *ctx.args)
            gs, gb = cloth.backward(grad_out)
            return gs.to(stretch.dtype), gb.to(bend.dtype), None, None, None, None

    return XpbdRollout


_FN = None


def rollout(stretch, bend, cloth: DiffCloth, frames: int, substeps: int = 10, iterations: int = 2):
    """Differentiable final positions of `cloth` (autograd through the
    library's adjoint)."""
    global _FN
    if _FN is None:
        _FN = _autograd_function()
    return _FN.apply(stretch, bend, cloth, frames, substeps, iterations)
