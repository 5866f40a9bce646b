"""Test infrastructure only: a float64 PyTorch restatement of the
contact-free XPBD rollout, for checking the library's hand-written adjoint
against automatic differentiation and finite differences.  Nothing in the
product imports it.

It restates the same schedule and arithmetic as the solver for a cloth
without contacts (native/src/ssbl_xpbd_cuda_abi41.cu: prediction 1869-1925,
stretch 1927-1980 as a snapshot gather, pins 3466-3509, bends by colour
2886-2970, velocity 5846-5884, order 9165-9376), in float64 with torch ops so
that autograd yields a reference gradient with respect to per-constraint
compliances.  Branch decisions (caps, clamps, sign tests) are taken in
float64, so near a threshold they may differ from the float32 solver.

Every operation works on leading batch dimensions: compliance tensors of
shape (..., E) and (..., B) roll out states of shape (..., V, 3), so many
parameter sets (the perturbations of a finite-difference check) run as one
rollout, on any torch device.
"""
from __future__ import annotations

import numpy as np
import torch

EPS = 1.0e-7


def frame_ops(substeps: int, iterations: int, bends: bool) -> list:
    ops = []
    for s in range(substeps):
        ops.append(("predict", ()))
        for _ in range(1, iterations):
            ops.append(("pass", ("gather", "pin")))
        if s == substeps - 1 and bends:
            ops.append(("pass", ("gather",)))
            ops.append(("bends", ()))
            ops.append(("pass", ("pin", "velocity")))
        else:
            ops.append(("pass", ("gather", "pin", "velocity")))
    return ops


class Rollout:
    def __init__(self, cloth, options, dtype=torch.float64, device="cpu"):
        t = lambda a: torch.as_tensor(np.asarray(a, np.float64)).to(device=device, dtype=dtype)  # noqa: E731
        self.rest = t(cloth.positions_world)
        self.w = t(np.maximum(cloth.inv_mass, 0.0))
        self.V = len(self.rest)
        e = np.asarray(cloth.edges, np.int64).reshape(-1, 2)
        self.ei, self.ej = torch.as_tensor(e[:, 0], device=device), torch.as_tensor(e[:, 1], device=device)
        self.erest = t(cloth.edge_rest_lengths)
        # every vertex's incident edges (edge index, endpoint side) padded to
        # the largest degree: the stretch pass sums a vertex's corrections in
        # this fixed order, so the rollout is deterministic on any device
        # (an atomic index_add on a GPU sums in arrival order)
        V = len(cloth.positions_world)
        verts = np.concatenate([e[:, 0], e[:, 1]])
        slots = np.concatenate([np.arange(len(e)), np.arange(len(e)) + len(e)])  # i side: k, j side: E + k
        order = np.lexsort((slots, verts))
        verts, slots = verts[order], slots[order]
        deg = np.bincount(verts, minlength=V)
        width = max(int(deg.max()) if len(deg) else 0, 1)
        rank = np.arange(len(verts)) - np.repeat(np.cumsum(deg) - deg, deg)
        inc = np.full((V, width), 2 * len(e), np.int64)  # padding points at a zero row
        inc[verts, rank] = slots
        self.inc = torch.as_tensor(inc, device=device)
        b = np.asarray(cloth.bends, np.int64).reshape(-1, 2)
        self.bi, self.bj = torch.as_tensor(b[:, 0], device=device), torch.as_tensor(b[:, 1], device=device)
        self.brest = t(cloth.bend_rest_lengths)
        self.colors = [int(x) for x in cloth.bend_color_offsets]
        self.pinned = torch.zeros(self.V, dtype=torch.bool, device=device)
        self.target = torch.zeros(self.V, 3, dtype=dtype, device=device)
        for idx, pos, wt in zip(cloth.pin_indices, cloth.pin_targets_world, cloth.pin_weights):
            if wt >= 0.75:
                self.pinned[int(idx)] = True
                self.target[int(idx)] = t(pos)
        o = options
        self.damping = float(min(max(o.damping, 0.0), 1.0))
        self.gravity = t(o.gravity)
        self.thickness = float(o.cloth_thickness)
        self.dt_frame = float(o.dt)

    def _stretch(self, p, prev, k, dt):
        wi, wj = self.w[self.ei], self.w[self.ej]
        W = wi + wj
        live = W > 0
        delta = p[..., self.ej, :] - p[..., self.ei, :]
        length = torch.sqrt(torch.clamp((delta * delta).sum(-1), min=EPS))
        c = length - self.erest
        alpha = torch.clamp(k, min=0.0) / max(dt * dt, EPS)
        dl = -c / torch.where(live, W + alpha, torch.ones_like(W))
        corr = delta * (0.18 * dl / torch.clamp(length, min=EPS))[..., None]
        clen = torch.sqrt(torch.clamp((corr * corr).sum(-1), min=1e-30))
        maxc = torch.clamp(torch.clamp(torch.clamp(self.erest, min=0.0) * 0.10, max=0.025), min=0.0025)
        capped = clen > maxc
        corr = torch.where(capped[..., None], corr * (maxc / torch.clamp(clen, min=EPS))[..., None], corr)
        corr = corr * live[:, None]
        di = -corr * wi[:, None]
        dj = corr * wj[:, None]
        kp = torch.where(c > 0, torch.full_like(c, 0.08), torch.zeros_like(c))[..., None]
        both = torch.cat([di, dj, torch.zeros_like(di[..., :1, :])], -2)  # (..., 2E + 1, 3)
        both_prev = torch.cat([di * kp, dj * kp, torch.zeros_like(di[..., :1, :])], -2)
        p = p + both[..., self.inc, :].sum(-2)
        prev = prev + both_prev[..., self.inc, :].sum(-2)
        return p, prev

    def _bends(self, p, prev, k, dt):
        for c0, c1 in zip(self.colors[:-1], self.colors[1:]):
            if c1 <= c0:
                continue
            sl = slice(c0, c1)
            i, j, rest, kk = self.bi[sl], self.bj[sl], self.brest[sl], k[..., sl]
            wi, wj = self.w[i], self.w[j]
            W = wi + wj
            delta = p[..., j, :] - p[..., i, :]
            len_sq = (delta * delta).sum(-1)
            ok = (W > 0) & (rest > EPS) & (len_sq > 1.0e-10)
            inv_len = 1.0 / torch.sqrt(torch.where(ok, len_sq, torch.ones_like(len_sq)))
            length = len_sq * inv_len
            c = length - rest
            ok = ok & (torch.abs(c) > 1.0e-6)
            alpha = torch.clamp(kk, min=0.0) / max(dt * dt, EPS)
            dl = -c / torch.clamp(W + alpha, min=EPS)
            corr = delta * (0.10 * dl * inv_len)[..., None]
            clen = torch.sqrt(torch.clamp((corr * corr).sum(-1), min=1e-30))
            maxc = torch.clamp(torch.clamp(torch.clamp(rest, min=self.thickness) * 0.08, max=0.020), min=2.5e-4)
            capped = clen > maxc
            corr = torch.where(capped[..., None], corr * (maxc / torch.clamp(clen, min=EPS))[..., None], corr)
            corr = corr * ok[..., None]
            di, dj = -corr * wi[:, None], corr * wj[:, None]
            p = p.index_add(-2, i, di).index_add(-2, j, dj)
            prev = prev.index_add(-2, i, di * 0.06).index_add(-2, j, dj * 0.06)
        return p, prev

    def _velocity(self, p, prev, vel, dt):
        sdt = max(dt, EPS)
        free = (self.w > 0)[:, None]
        measured = (p - prev) * (1.0 / sdt)
        proj = measured - vel
        pdb = (proj * vel).sum(-1)
        scale = torch.where(pdb > 0, torch.full_like(pdb, 0.9), torch.ones_like(pdb))[..., None]
        fb = proj * scale
        fspeed = torch.sqrt(torch.clamp((fb * fb).sum(-1), min=1e-30))
        max_speed = max(2.0e-4, max(self.thickness, 0.0) * 0.35) / sdt
        clamp = (scale[..., 0] < 1.0) & (fspeed > max_speed) & (fspeed > EPS)
        fb = torch.where(clamp[..., None], fb * (max_speed / torch.clamp(fspeed, min=EPS))[..., None], fb)
        return torch.where(free, vel + fb, torch.zeros_like(vel))

    def frame(self, p, prev, vel, stretch_k, bend_k, substeps: int, iterations: int):
        """One frame from the state (p, prev, vel); returns the next state."""
        dt = self.dt_frame / substeps
        free = (self.w > 0)[:, None]
        pin = self.pinned[:, None]
        ops = frame_ops(substeps, iterations, len(self.colors) > 1 and self.colors[-1] > 0)
        for kind, flags in ops:
            if kind == "predict":
                prev = p
                vf = (vel + self.gravity * dt) * self.damping
                pf = p + vf * dt
                p = torch.where(free, pf, self.rest)
                vel = torch.where(free, vf, torch.zeros_like(vf))
                p = torch.where(pin, self.target, p)
                prev = torch.where(pin, self.target, prev)
                vel = torch.where(pin, torch.zeros_like(vel), vel)
            elif kind == "pass":
                if "gather" in flags:
                    p, prev = self._stretch(p, prev, stretch_k, dt)
                if "pin" in flags:
                    p = torch.where(pin, self.target, p)
                    prev = torch.where(pin, self.target, prev)
                    vel = torch.where(pin, torch.zeros_like(vel), vel)
                if "velocity" in flags:
                    vel = self._velocity(p, prev, vel, dt)
            else:
                p, prev = self._bends(p, prev, bend_k, dt)
        return p, prev, vel

    def run(self, stretch_k, bend_k, frames: int, substeps: int, iterations: int):
        batch = torch.broadcast_shapes(stretch_k.shape[:-1], bend_k.shape[:-1])
        p = self.rest.expand(*batch, self.V, 3).clone()
        prev = p.clone()
        vel = torch.zeros_like(p)
        for _ in range(frames):
            p, prev, vel = self.frame(p, prev, vel, stretch_k, bend_k, substeps, iterations)
        return p
