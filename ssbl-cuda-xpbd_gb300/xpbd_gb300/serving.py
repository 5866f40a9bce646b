"""Serving form: a request loop that runs many cloth solves on one GPU.

Requests (a cloth, its solver options and colliders, a horizon in frames)
arrive over time.  The engine admits them while their device memory fits a
budget, keeps their state resident on the device until the horizon is
reached, and advances every resident request by one frame per tick
(continuous batching: requests join and leave between ticks, never waiting
for a whole batch to drain).

Solvers of newly admitted requests are built (CSR builds, uploads, static
SDF, frame-graph capture) on worker threads while the resident requests keep
stepping; a cohort joins the ticks once its solver is ready.  Requests
admitted in the same tick with the same substeps / iterations form a
cohort: cloths under ``group_below`` vertices share one batched solver (one
launch sequence, one CUDA graph per frame), larger ones get a solver of
their own.  Every cohort has its own CUDA stream and all cohorts' frames are
launched before any is waited on, so their work overlaps on the device.  A
finished request is downloaded and switched inactive (its cloth is skipped by
every kernel); a cohort's memory returns to the budget when its last request
finishes.  A cloth's result does not depend on the cohort it runs in: each
cloth of a batched solver is stepped exactly as it is stepped alone.

Latency-aware admission.  A request's frame latency is the duration of the
tick that advances it, and a tick advances every resident request, so the
tick time follows the resident work (vertex-substeps per tick) divided by
the device's throughput.  With ``frame_latency_ms`` set, a request is
admitted only while the resident work plus its own stays within the work one
tick can do in ``latency_headroom`` (default 0.9) of that time at the
throughput measured over recent ticks (exponential average of
vertex-substeps per second of tick time, seeded by ``rate_guess``); the rest
waits in the queue in arrival order.  The headroom absorbs the tick-to-tick
variation of the measured rate, so the 99th percentile of frame latency
stays under the target rather than around it.  Without a
target, admission is by device memory alone.

The solver back end is injectable (``backend``) so the scheduling logic can
be exercised without a GPU.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .scene import ClothData, SolverOptions


@dataclass
class ClothRequest:
    cloth: ClothData
    options: SolverOptions
    static_triangles: np.ndarray
    frames: int
    substeps: int = 10
    iterations: int = 2
    request_id: int = -1
    arrival: float = 0.0  # seconds on the engine clock


@dataclass
class RequestResult:
    request_id: int
    positions: np.ndarray
    frames: int
    vertices: int
    arrival: float
    admitted: float
    finished: float
    frame_latency_ms: list = field(default_factory=list)


def estimate_device_bytes(req: ClothRequest) -> int:
    """Upper estimate of a request's device memory, from its sizes and the
    allocation rules of the solver (state rows, constraint CSRs, pins, the
    self-collision tables with 64 cells per triangle / edge and 64 member
    slots per edge-hash bucket, static SDF)."""
    c, o = req.cloth, req.options
    V, E, T = len(c.positions_world), len(c.edges), len(c.triangles)
    B, L = len(c.bends), len(c.lra_edges)
    b = V * (16 * 5 + 4 + 16 + 4 * 2 + 12 + 4 * 2) + E * (8 + 4 + 16) + T * 16 + B * 12 + L * 16 + 4 * 8
    b += 8 * 64 + 4096  # bend colour ranges and recorded fused-frame operations
    if o.self_collision:
        def pow2(x):
            return 1 << max(int(math.ceil(math.log2(max(x, 1)))), 0)

        vb = pow2(max(1024, 4 * V)) if V >= 128 else 0
        tb = pow2(max(1024, 4 * T)) if T >= 64 else 0
        eb = pow2(max(1024, 4 * E)) if E >= 64 else 0
        b += V * (4 + 4 * 32 + 32 + 16 + 4) + (vb + tb + eb) * 8 + T * 64 * 4 + E * 64 * 4 + 3 * (max(vb, tb, eb) // 4096 + 2) * 4
        b += 3 * max(vb, tb, eb) * 4 + 3 * 4  # lists of buckets of more than 32 members
        # edge hash: 64 member slots per bucket, overflow bits, list and region
        # starts, the record of insertions past the slots (8 B each)
        if eb:
            b += eb * 64 * 4 + (eb // 32 + 1) * 4 + 2 * (min(eb, E * 64 // 65 + 1) + 1) * 4
            b += min(E * 64, max(1 << 20, E)) * 8 + 8
    if o.stretch_optimization_enabled:
        # CG blocks, preconditioner, r / z / d / q, cap sums, off-diagonal per
        # stretch-CSR entry (two per edge), colour-sorted cap edges, partials
        b += V * (32 + 32 + 4 * 16 + 16) + E * (2 * 16 + 12) + (V // 256 + 1) * 36 + 1024
    nst = len(req.static_triangles)
    if nst:
        res = max(o.static_sdf_max_resolution if o.static_sdf_max_resolution > 0 else 160, 16)
        b += res ** 3 * 4 + nst * 48
    return int(b * 1.05) + (1 << 16)


class NativeBackend:
    """Cohort solvers on the GB300 library."""

    def __init__(self):
        from . import native

        self.native = native

    def create(self, reqs: list):
        if len(reqs) == 1:
            r = reqs[0]
            return self.native.NativeXpbdSolver(r.cloth, r.options, r.static_triangles)
        return self.native.NativeXpbdBatch([(r.cloth, r.options, r.static_triangles) for r in reqs])

    @staticmethod
    def prepare(solver, substeps, iterations):
        solver.prepare_graph(substeps, iterations)

    @staticmethod
    def device_bytes(solver) -> int:
        return solver.device_bytes()

    @staticmethod
    def step(solver, substeps, iterations):
        solver.step(substeps, iterations, diagnostics=False, synchronize=False)

    @staticmethod
    def wait(solver):
        solver.synchronize()

    @staticmethod
    def download(solver, slot: int, batched: bool) -> np.ndarray:
        return solver.download_cloth_positions(slot) if batched else solver.download_positions().copy()

    @staticmethod
    def deactivate(solver, slot: int, batched: bool):
        if batched:
            solver.set_cloth_active(slot, False)

    @staticmethod
    def close(solver):
        solver.close()


class _Cohort:
    def __init__(self, solver, reqs, admitted, nbytes, batched):
        self.solver = solver
        self.reqs = reqs
        self.done = [0] * len(reqs)
        self.live = [True] * len(reqs)
        self.admitted = admitted
        self.bytes = nbytes
        self.batched = batched
        self.latency = [[] for _ in reqs]
        self.substeps = reqs[0].substeps
        self.iterations = reqs[0].iterations


class ServingEngine:
    """Continuous-batching request loop under a device-memory budget."""

    def __init__(self, hbm_budget_bytes: int, group_below: int = 50_000, max_cohort_vertices: int = 2_000_000,
                 max_admit_per_tick: int = 64, backend=None, clock=time.perf_counter, workers: int = 4,
                 frame_latency_ms: float | None = None, rate_guess: float = 2.0e8, latency_headroom: float = 0.9):
        self.budget = int(hbm_budget_bytes)
        self.frame_latency_ms = frame_latency_ms
        self.latency_headroom = float(latency_headroom)
        self.rate = float(rate_guess)     # vertex-substeps per second of tick time (measured)
        self.resident_work = 0            # vertex-substeps per tick of admitted requests
        self.workers = workers
        self.pool = None
        if workers > 0:
            from concurrent.futures import ThreadPoolExecutor

            self.pool = ThreadPoolExecutor(max_workers=workers)
        self.building: list = []  # (future, reqs, reserved bytes)
        self.group_below = group_below
        self.max_cohort_vertices = max_cohort_vertices
        self.max_admit_per_tick = max_admit_per_tick
        self.backend = backend if backend is not None else NativeBackend()
        self.clock = clock
        self.queue: deque = deque()
        self.cohorts: list[_Cohort] = []
        self.used_bytes = 0
        self.peak_bytes = 0
        self.t0 = None
        self.completed_vertex_substeps = 0
        self.ticks = 0

    # ---------------------------------------------------------------- API
    def now(self) -> float:
        if self.t0 is None:
            self.t0 = self.clock()
        return self.clock() - self.t0

    def submit(self, req: ClothRequest) -> None:
        if req.frames <= 0:
            raise ValueError("request horizon must be at least one frame")
        self.queue.append(req)

    @property
    def live_requests(self) -> int:
        return sum(sum(c.live) for c in self.cohorts)

    def idle(self) -> bool:
        return not self.queue and not self.cohorts and not self.building

    def close(self) -> None:
        """Wait for solvers being built, then free every solver."""
        for fut, _, _ in self.building:
            try:
                self.backend.close(fut.result())
            except Exception:
                pass
        self.building = []
        for c in self.cohorts:
            self.backend.close(c.solver)
        self.cohorts = []
        self.used_bytes = 0
        self.resident_work = 0
        if self.pool is not None:
            self.pool.shutdown(wait=True)
            self.pool = None

    def tick(self) -> list[RequestResult]:
        """Admit what fits, advance every resident request by one frame,
        retire finished requests.  Returns the requests finished now."""
        self.ticks += 1
        self._admit()
        self._collect_built(wait=not self.cohorts)
        if not self.cohorts:
            return []
        starts = []
        for c in self.cohorts:
            starts.append(self.clock())
            self.backend.step(c.solver, c.substeps, c.iterations)
        finished = []
        tick_work = 0
        for c, t_launch in zip(self.cohorts, starts):
            self.backend.wait(c.solver)
            lat = (self.clock() - t_launch) * 1000.0
            for k, r in enumerate(c.reqs):
                if not c.live[k]:
                    continue
                c.done[k] += 1
                c.latency[k].append(lat)
                work = len(r.cloth.positions_world) * r.substeps
                self.completed_vertex_substeps += work
                tick_work += work
                if c.done[k] >= r.frames:
                    finished.append(self._retire(c, k))
        tick_s = self.clock() - starts[0]
        if tick_work > 0 and tick_s > 0:
            self.rate = 0.8 * self.rate + 0.2 * (tick_work / tick_s)
        for c in [c for c in self.cohorts if not any(c.live)]:
            self.backend.close(c.solver)
            self.used_bytes -= c.bytes
            self.cohorts.remove(c)
        return finished

    def run(self, requests: list[ClothRequest], duration: float | None = None, drain: bool = False) -> dict:
        """Feed `requests` by arrival time (engine clock), ticking until
        `duration` seconds have passed (and, with `drain`, until every
        admitted and queued request is done).  Returns the statistics."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        results: list[RequestResult] = []
        self.now()
        while True:
            t = self.now()
            while pending and pending[0].arrival <= t:
                self.submit(pending.popleft())
            if duration is not None and t >= duration and not drain:
                break
            if self.idle():
                if not pending:
                    break
                if duration is not None and pending[0].arrival > duration and not drain:
                    break
                time.sleep(max(0.0, min(pending[0].arrival - t, 0.01)))
                continue
            results += self.tick()
        return self.stats(results, self.now())

    def stats(self, results: list[RequestResult], elapsed: float) -> dict:
        lat = [x for r in results for x in r.frame_latency_ms]
        for c in self.cohorts:  # frames of requests still running count too
            for k in range(len(c.reqs)):
                lat += c.latency[k]
        queue_delay = [r.admitted - r.arrival for r in results]
        return {
            "elapsed_s": elapsed,
            "ticks": self.ticks,
            "completed_requests": len(results),
            "resident_requests": self.live_requests,
            "queued_requests": len(self.queue),
            "vertex_substeps": self.completed_vertex_substeps,
            "throughput": self.completed_vertex_substeps / elapsed if elapsed > 0 else 0.0,
            "frame_latency_ms_p50": float(np.percentile(lat, 50)) if lat else None,
            "frame_latency_ms_p99": float(np.percentile(lat, 99)) if lat else None,
            "frames": len(lat),
            "queue_delay_s_p50": float(np.percentile(queue_delay, 50)) if queue_delay else None,
            "queue_delay_s_p99": float(np.percentile(queue_delay, 99)) if queue_delay else None,
            "peak_device_bytes": self.peak_bytes,
            "budget_bytes": self.budget,
            "frame_latency_target_ms": self.frame_latency_ms,
            "measured_rate": self.rate,
            "results": results,
        }

    # ----------------------------------------------------------- internals
    def _admit(self) -> None:
        """FIFO admission: requests leave the queue in arrival order while
        their estimated memory fits the budget; small ones admitted together
        share a cohort."""
        admitted: list[ClothRequest] = []
        reserve = 0
        work_cap = (None if self.frame_latency_ms is None
                    else self.latency_headroom * self.rate * self.frame_latency_ms / 1000.0)
        while self.queue and len(admitted) < self.max_admit_per_tick:
            need = estimate_device_bytes(self.queue[0])
            if self.used_bytes + reserve + need > self.budget:
                if not self.cohorts and not self.building and not admitted and reserve == 0:
                    raise MemoryError(f"request {self.queue[0].request_id} needs {need} bytes, over the whole budget")
                break
            work = len(self.queue[0].cloth.positions_world) * self.queue[0].substeps
            if work_cap is not None and self.resident_work > 0 and self.resident_work + work > work_cap:
                break  # one tick would take longer than the frame-latency target
            reserve += need
            self.resident_work += work
            admitted.append(self.queue.popleft())
        if not admitted:
            return
        t = self.now()
        groups: dict[tuple, list] = {}
        for r in admitted:
            if len(r.cloth.positions_world) >= self.group_below:
                self._open([r], t)
            else:
                groups.setdefault((r.substeps, r.iterations), []).append(r)
        for reqs in groups.values():
            part, verts = [], 0
            for r in reqs:
                v = len(r.cloth.positions_world)
                if part and verts + v > self.max_cohort_vertices:
                    self._open(part, t)
                    part, verts = [], 0
                part.append(r)
                verts += v
            if part:
                self._open(part, t)

    def _build(self, reqs: list):
        solver = self.backend.create(reqs)
        prepare = getattr(self.backend, "prepare", None)
        if prepare is not None:
            prepare(solver, reqs[0].substeps, reqs[0].iterations)
        return solver

    def _open(self, reqs: list, t: float) -> None:
        reserved = sum(estimate_device_bytes(r) for r in reqs)
        self.used_bytes += reserved
        self.peak_bytes = max(self.peak_bytes, self.used_bytes)
        if self.pool is None:
            self._join(self._build(reqs), reqs, reserved)
        else:
            self.building.append((self.pool.submit(self._build, reqs), reqs, reserved))

    def _join(self, solver, reqs: list, reserved: int) -> None:
        nbytes = self.backend.device_bytes(solver)
        self.used_bytes += nbytes - reserved
        self.peak_bytes = max(self.peak_bytes, self.used_bytes)
        self.cohorts.append(_Cohort(solver, reqs, self.now(), nbytes, batched=len(reqs) > 1))

    def _collect_built(self, wait: bool) -> None:
        """Move solvers that finished building into the ticks (waiting for
        the first one when nothing else would run)."""
        if not self.building:
            return
        if wait:
            from concurrent.futures import FIRST_COMPLETED
            from concurrent.futures import wait as fwait

            fwait([f for f, _, _ in self.building], return_when=FIRST_COMPLETED)
        still = []
        for fut, reqs, reserved in self.building:
            if fut.done():
                self._join(fut.result(), reqs, reserved)
            else:
                still.append((fut, reqs, reserved))
        self.building = still

    def _retire(self, c: _Cohort, k: int) -> RequestResult:
        r = c.reqs[k]
        self.resident_work -= len(r.cloth.positions_world) * r.substeps
        pos = self.backend.download(c.solver, k, c.batched)
        self.backend.deactivate(c.solver, k, c.batched)
        c.live[k] = False
        return RequestResult(r.request_id, pos, c.done[k], len(r.cloth.positions_world), r.arrival, c.admitted,
                             self.now(), c.latency[k])
