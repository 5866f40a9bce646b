#!/usr/bin/env python3
"""Benchmark of the GB300 XPBD cloth step (vertex-substeps/s).

Workloads (a "step" is one frame of 10 substeps x 2 iterations):

* ``batch256`` (default): 256 independent cloths, sides drawn uniformly from
  16-128 vertices (1,589,788 vertices in all), stretch and bend compliance
  log-uniform in [1e-8, 1e-4], 2-8 random hard pins per cloth, fast or
  strict self collision (2 mm) with probability 0.5, a sphere and the ground;
  all cloths run in one batched solver (one launch sequence per frame,
  captured as one CUDA graph).  The same cloths are also run the plain way,
  one ABI41 handle per cloth stepped back to back, and reported as ``plain``.
* ``drop10k``: a 100 x 100 cloth (10,000 vertices) with seeded +-1 mm jitter
  dropped onto a sphere (r = 0.3 m) and a 64^3 static SDF of a box and a
  torus, strict self collision with 2 mm thickness, friction 0.3.
* ``plain32``: 32 x 32 grid, two pinned corners, ground plane.

Inputs are seeded synthetic (the reference uses no dataset).

Timing: W untimed warm-up frames, then K frames, each bracketed by CUDA
events on the solver's own stream; before every timed frame a 256 MiB buffer
is written on that stream so L2 (129 MB) starts cold.  ``value`` = vertices x
substeps x K x N / time.

Also reported: ``e2e`` through the C-ABI with host buffers (pin targets
uploaded, positions downloaded every frame), the per-kernel profile of one
un-graphed frame and the roofline of the dominant kernel kind, SM clocks
sampled during the timed region, and the CPU oracle timed on a bounded
sample of the same workload.

Also in the default line (``--extras 1``): the plain32 and drop10k
workloads device-timed the same way; the serving loop over 60 s of Poisson
arrivals with its p50 / p99 frame latency under a frame-latency target
(``--serve-latency-ms``, default 100); the differentiable rollout + adjoint;
and ``reference_gpu``, the reference's own CUDA solver (built unchanged for
sm_103a from its sources by oracle/build_ref.py) stepping the same 256 cloths
one handle at a time on the default stream, one wait per frame, as the add-on
does: the plain baseline of the batched form; and ``reference_gpu_plain32`` /
``reference_gpu_drop10k``, the same solver on the two single-cloth workloads
(one handle, one wait per frame), beside which ``plain32_over_reference`` and
``drop10k_over_reference`` give this repository's ratio.

``--impl reference``: the reference's step has no CPU implementation, so that
arm times the CPU restatement of the reference's algorithm (oracle/) with
all host threads, on every 16th cloth of the workload per step; its scenes
come from the pure-Python builders, so it loads no library of this
repository.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ssbl-cuda-xpbd_gb300"))

import numpy as np  # noqa: E402

from xpbd_gb300 import scene  # noqa: E402

METRIC = "vertex-substeps/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
F3 = 12  # bytes of a position / velocity row read or written (x, y, z f32)

DESCRIPTIONS = {
    "batch256": "256 independent cloths, side U{16..128} verts (1,589,788 verts), compliance log-uniform 1e-8..1e-4, "
                "2-8 hard pins each, fast/strict self collision (2 mm, p=0.5), sphere + ground, one batched solver "
                "(one CUDA graph per frame), 10 substeps x 2 iterations per frame",
    "drop10k": "10k cloth (100x100 grid, 19,602 tris) dropped on a sphere + 64^3 box/torus SDF, strict self "
               "collision 2 mm, friction 0.3, 10 substeps x 2 iterations per frame",
    "plain32": "plain 32x32 grid (1,024 verts), two pinned corners, ground, 10 substeps x 2 iterations",
    "diff": "differentiable: 64x64 cloth (4,096 verts), per-constraint stretch / bend compliance fields, no contacts, "
            "60 frames x 10 substeps x 2 iterations; one step = rollout + adjoint (per-frame checkpoints) of L2 to a "
            "target from another seeded compliance field",
    "serve": "serving: Poisson arrivals 200/s of cloth solves, V log-uniform 1k-250k (16 grid sizes), horizons "
             "30-240 frames, random sphere and/or box/torus SDF, strict self collision 2 mm, admitted by a "
             "device-memory budget, resident until done, one frame per resident request per tick",
    "prep": "input preprocessing: constraint inputs of a 500x500 cloth (250,000 verts, 498,002 tris, jittered, "
            "2 hard pins + hidden tethers) from host arrays to host arrays; edges, bend pairs, rest lengths and "
            "inverse masses on the device, greedy colouring and tethers on the host",
}


def workload(name: str, cloths: int = 256) -> list:
    if name == "batch256":
        return scene.batched_scenes(cloths, seed=0, frames=120)
    if name == "drop10k":
        return [scene.drop_scene(100, 200, seed=0, self_mode=2)]
    if name == "plain32":
        return [scene.plain_grid_scene(32, 120)]
    if name in ("serve", "diff"):
        return []
    raise SystemExit(f"unknown workload {name}")


def algorithmic_bytes(kind: str, V: int, E: int, T: int, B: int, counters: dict) -> float | None:
    """Compulsory bytes of one launch of a kernel kind, by the per-kernel
    model of the cloth step (12 B per position / velocity row read or
    written):
      predict              52 B per vertex (read x, v, w; write x, prev)
      stretch pass         12 B per edge + 24 B per vertex (constraint stream,
                           x read and written) + 36 B per vertex for the
                           contact stages fused into the same pass
      velocity pass        52 B per vertex
      bend colour          12 B per bend + 2 endpoints read and written
      vertex-triangle /    12 B per candidate gather: the candidate's row,
      edge-edge query      per evaluated bucket slot (vertex-triangle) or per
                           visited slot whose candidate id is above the query
                           edge's (edge-edge: a pair is evaluated from its
                           lower edge, so the other slots end at the id);
                           counted in the profiled frames
      hash build           12 B per primitive row read, 32 B per entry (key
                           and id through a two-pass sort, read and written),
                           8 B per bucket (cell start / end)
    Returns None for kinds without a model."""
    if kind == "predict":
        return 52.0 * V
    if kind == "stretch_pass":
        return 12.0 * E + 24.0 * V + 36.0 * V
    if kind == "vertex_pass":
        return 52.0 * V
    if kind == "bend_color":
        return 12.0 * B + 48.0 * B
    if kind == "edge_edge" and counters.get("ee_gathers"):
        return 12.0 * counters["ee_gathers"]
    if kind == "vertex_triangle" and counters.get("vt_slots"):
        return 12.0 * counters["vt_slots"]
    if kind == "edge_hash" and counters.get("edge_entries"):
        return 2 * F3 * counters["edge_hashed"] + 32.0 * counters["edge_entries"] + 8.0 * counters["edge_buckets"]
    if kind == "triangle_hash" and counters.get("tri_entries"):
        return 3 * F3 * counters["tri_hashed"] + 32.0 * counters["tri_entries"] + 8.0 * counters["tri_buckets"]
    return None


def full_gather_bytes(kind: str, counters: dict) -> float | None:
    """What a query evaluation actually loads, beside the per-gather model:
    per item its own indices and rows and its bucket range, per visited slot
    the candidate id, per gathered candidate its indices and rows (40 B per
    edge-edge item, 4 B per slot and 32 B per gather; 20 + 52 B per
    vertex-triangle slot)."""
    if kind == "edge_edge" and counters.get("ee_items"):
        return ((8 + 2 * F3 + 8) * counters["ee_items"] + 4 * counters["ee_slots"]
                + (8 + 2 * F3) * counters.get("ee_gathers", counters["ee_slots"]))
    if kind == "vertex_triangle" and counters.get("vt_items"):
        return (F3 + 8) * counters["vt_items"] + (4 + 12 + 3 * F3) * counters["vt_slots"]
    return None


# DRAM bytes (read + write) per visited bucket slot of the edge-edge query
# passes: dram__bytes_read.sum + dram__bytes_write.sum of every edge-edge
# launch of one profiled frame of the 64-cloth batch under ncu (cold caches:
# ncu flushes them before each launch), divided by the slots that frame
# evaluated (`--profile-frame`); scaled by the slots of the measured workload.
EE_DRAM_BYTES_PER_SLOT = 14.4
# ... and per insertion of an edge-hash build (slot insertion, overflow
# kernels, trim and bucket ordering) from the same capture: the frame's last
# build over its insertions.
EDGE_HASH_DRAM_BYTES_PER_ENTRY = 20.2


def measured_traffic(kind: str, counters: dict, launches: int) -> float | None:
    """DRAM traffic per launch of a kernel kind, scaled from an ncu capture
    of a smaller case, or None where none was taken."""
    if kind == "edge_edge" and counters.get("ee_slots") and launches > 0:
        return EE_DRAM_BYTES_PER_SLOT * counters["ee_slots"] / launches
    if kind == "edge_hash" and counters.get("edge_entries"):
        return EDGE_HASH_DRAM_BYTES_PER_ENTRY * counters["edge_entries"]  # one build
    return None


def peaks() -> tuple[float, str]:
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def sample_indices(count: int, stride: int = 16) -> list:
    """Evenly spaced cloths of a batched workload (every `stride`-th), the
    bounded sample the CPU timings step: the same mix of sizes and fast /
    strict self collision as the whole set."""
    return list(range(0, count, stride)) if count > 1 else [0]


def cpu_oracle_rate(scs: list, budget_s: float) -> tuple[float, int, str]:
    """The oracle (all host threads) stepping an evenly spaced sample of the
    workload's cloths one frame each, for about `budget_s` seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import xpbd_oracle

    threads = xpbd_oracle.set_threads(os.cpu_count() or 1)
    sample = [scs[k] for k in sample_indices(len(scs))]
    work, elapsed, cloths, frames_per = 0, 0.0, 0, 1 if len(scs) > 1 else 400
    n = 0
    for sc in sample:
        o = xpbd_oracle.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
        o.step(sc.substeps, sc.iterations)  # warm-up frame
        V = len(sc.cloth.positions_world)
        t0 = time.perf_counter()
        n = 0
        while n < frames_per:
            o.step(sc.substeps, sc.iterations)
            n += 1
            if elapsed + time.perf_counter() - t0 >= budget_s:
                break
        elapsed += time.perf_counter() - t0
        work += V * sc.substeps * n
        cloths += 1
        if elapsed >= budget_s:
            break
    if len(scs) > 1:
        what = (f"{cloths} cloths (every 16th of the workload's {len(scs)}), one warm-up frame then one timed frame "
                f"each, {elapsed:.1f} s")
    else:
        what = f"{n} frames after one warm-up frame, {elapsed:.1f} s"
    return work / elapsed, threads, what


def max_over_ranks(value: float, world: int) -> float:
    """The largest of every rank's value (the slowest replica's time), then a
    barrier; the value itself with one rank.  Works on the NCCL process group
    of the GPU runs (CUDA tensor) and on gloo (host tensor)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def run_reference(args, scs, world, rank):
    """Reference arm: the reference's step exists only as CUDA code, so this
    arm times its CPU restatement (oracle/) with all host threads, on an
    evenly spaced sample of the workload's cloths per step.  The scenes are
    built by the pure-Python builders: no library of this repository is
    loaded."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import xpbd_oracle

    threads = xpbd_oracle.set_threads(os.cpu_count() or 1)
    solvers = [xpbd_oracle.OracleSolver.from_scene(s.cloth, s.options, s.static_triangles) for s in scs]
    V = sum(len(s.cloth.positions_world) for s in scs)
    S, I = scs[0].substeps, scs[0].iterations
    for _ in range(args.warmup):
        for o in solvers:
            o.step(S, I)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for o in solvers:
            o.step(S, I)
    el = time.perf_counter() - t0
    value = V * S * args.steps / el
    what = (f"{len(scs)} of the workload's {args.batch_cloths} cloths (every 16th: sizes 16-128, fast and strict self "
            f"collision; {V} vertices) per step, one frame each" if args.workload == "batch256"
            else "the whole workload, one frame per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": DESCRIPTIONS[args.workload], "vertices_per_step": V, "substeps": S, "iterations": I},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": what},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's step exists only as CUDA code; this arm is the C restatement of its algorithm on the host cores",
    }
    print(json.dumps(line), flush=True)


def device_time(solver, S: int, I: int, steps: int, torch, world: int = 1, clocks=None) -> float:
    """K frames, each bracketed by CUDA events on the solver's stream after a
    256 MiB write on that stream (L2 starts cold); returns the summed
    milliseconds (max over ranks)."""
    stream = torch.cuda.ExternalStream(solver.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        events[k][0].record(stream)
        solver.step(S, I, diagnostics=False, synchronize=False)
        events[k][1].record(stream)
    torch.cuda.synchronize()
    return max_over_ranks(sum(a.elapsed_time(b) for a, b in events), world)


def time_single(native, torch, name: str, steps: int, warmup: int) -> dict:
    """One of the single-cloth workloads (plain32, drop10k), device-timed."""
    sc = workload(name)[0]
    solver = native.NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    S, I = sc.substeps, sc.iterations
    for _ in range(warmup):
        solver.step(S, I, diagnostics=False, synchronize=False)
    ms = device_time(solver, S, I, steps, torch)
    launches = solver.last_step_launches()
    solver.close()
    V = len(sc.cloth.positions_world)
    return {"value": V * S * steps / (ms / 1000.0), "unit": METRIC, "ms_per_step": ms / steps, "frames": steps,
            "launches_per_step": launches, "workload": DESCRIPTIONS[name]}


def time_reference_gpu(scs, frames: int, torch) -> dict:
    """The reference's own CUDA solver (native/src/ssbl_xpbd_cuda_abi41.cu,
    built unchanged with its own flags for sm_103a by oracle/build_ref.py)
    on the same cloths, the way the add-on steps them: one handle per cloth,
    each step(diagnostics=False, synchronize=False) in turn on the default
    stream, one device wait per frame (session_manager.py:2528-2591)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_solver

    if not ref_solver.available():
        return {"unavailable": "reference solver not built (oracle/build_ref.py needs the reference sources)"}
    solvers = [ref_solver.RefSolver.from_scene(s) for s in scs]
    S, I = scs[0].substeps, scs[0].iterations
    V = sum(len(s.cloth.positions_world) for s in scs)
    for r in solvers:
        r.step(S, I, diagnostics=False, synchronize=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(frames):
        for r in solvers:
            r.step(S, I, diagnostics=False, synchronize=False)
        torch.cuda.synchronize()
    el = time.perf_counter() - t0
    for r in solvers:
        r.close()
    return {"value": V * S * frames / el, "unit": METRIC, "ms_per_step": 1000.0 * el / frames, "frames": frames,
            "handles": len(scs), "what": "reference CUDA solver, one handle per cloth on the default stream, "
            "one wait per frame (host-timed)"}


def time_reference_single(name: str, frames: int, warmup: int, torch) -> dict:
    """The reference's own CUDA solver on one of the single-cloth workloads
    (plain32, drop10k), stepped as the add-on steps a cloth: step(diagnostics
    =False, synchronize=False) on the default stream, then a device wait
    (host-timed per frame, after `warmup` frames)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_solver

    if not ref_solver.available():
        return {"unavailable": "reference solver not built (oracle/build_ref.py needs the reference sources)"}
    sc = workload(name)[0]
    r = ref_solver.RefSolver.from_scene(sc)
    S, I = sc.substeps, sc.iterations
    for _ in range(warmup):
        r.step(S, I, diagnostics=False, synchronize=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(frames):
        r.step(S, I, diagnostics=False, synchronize=False)
        torch.cuda.synchronize()
    el = time.perf_counter() - t0
    r.close()
    V = len(sc.cloth.positions_world)
    return {"value": V * S * frames / el, "unit": METRIC, "ms_per_step": 1000.0 * el / frames, "frames": frames,
            "what": "reference CUDA solver, one handle, default stream, one wait per frame (host-timed)",
            "workload": DESCRIPTIONS[name]}


def time_plain(native, scs, frames: int) -> dict:
    """The plain drop-in: one ABI41 handle per cloth, stepped back to back
    (no per-handle sync) with one wait per frame, like the reference add-on
    steps its cloths."""
    solvers = [native.NativeXpbdSolver(s.cloth, s.options, s.static_triangles) for s in scs]
    S, I = scs[0].substeps, scs[0].iterations
    V = sum(len(s.cloth.positions_world) for s in scs)
    for _ in range(2):
        for s in solvers:
            s.step(S, I, diagnostics=False, synchronize=False)
        for s in solvers:
            s.synchronize()
    t0 = time.perf_counter()
    for _ in range(frames):
        for s in solvers:
            s.step(S, I, diagnostics=False, synchronize=False)
        for s in solvers:
            s.synchronize()
    el = time.perf_counter() - t0
    launches = sum(s.last_step_launches() for s in solvers)
    for s in solvers:
        s.close()
    return {"value": V * S * frames / el, "unit": METRIC, "ms_per_step": 1000.0 * el / frames, "frames": frames,
            "handles": len(scs), "launches_per_step": launches}


def run_prep(args, world, rank, local):
    """Input preprocessing of a 250k-vertex cloth: one step = one cloth's
    constraint inputs built from host arrays (scene.build_cloth with the
    device path), against the numpy restatement of the add-on's builder.
    The metric is vertices per second."""
    n = 500
    pos, tris = scene.grid_mesh(n, 5.0, 0.0)
    pos = (pos + np.random.default_rng(0).uniform(-1e-3, 1e-3, pos.shape)).astype(np.float32)
    w = np.zeros(len(pos), np.float32)
    w[[0, n - 1]] = 1.0
    V = len(pos)

    def numpy_build():
        return scene.build_cloth(pos, tris, 0.2, w, tether_slack=1.05)

    if args.impl == "reference":
        if rank != 0:
            return
        for _ in range(args.warmup):
            numpy_build()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            numpy_build()
        el = time.perf_counter() - t0
        value = V * args.steps / el
        print(json.dumps({"impl": "reference", "metric": "vertices/s", "value": value, "unit": "vertices/s",
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1000.0 * el / args.steps, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered grid)",
                          "config": {"workload": DESCRIPTIONS["prep"], "vertices": V, "triangles": len(tris)},
                          "cpu_baseline": {"value": value, "unit": "vertices/s", "cores": 1, "kind": "port",
                                           "sample": "the whole workload: numpy restatement of the builder"},
                          "e2e": {"value": value, "unit": "vertices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
              flush=True)
        return
    import torch

    torch.cuda.set_device(local)
    from xpbd_gb300 import build

    build.build()
    hard = w >= scene.PIN_HARD_WEIGHT_THRESHOLD
    for _ in range(args.warmup):
        scene.build_cloth(pos, tris, 0.2, w, tether_slack=1.05, device=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        scene.build_cloth(pos, tris, 0.2, w, tether_slack=1.05, device=True)
    el = time.perf_counter() - t0
    # the device step alone, and the numpy steps it replaces
    t1 = time.perf_counter()
    for _ in range(args.steps):
        scene.cloth_inputs_device(pos, tris, 0.2, hard)
    dev = (time.perf_counter() - t1) / args.steps
    t2 = time.perf_counter()
    scene.edge_constraints(tris, pos)
    scene.bend_constraints(tris, pos)
    scene.vertex_inverse_mass(pos, tris, 0.2, hard)
    ref_steps = time.perf_counter() - t2
    t3 = time.perf_counter()
    numpy_build()
    ref_full = time.perf_counter() - t3
    value = V * args.steps * world / el
    if rank != 0:
        return
    line = {
        "metric": "vertices/s", "value": value, "unit": "vertices/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered grid)",
        "config": {"workload": DESCRIPTIONS["prep"], "vertices": V, "triangles": len(tris), "parallelism": f"replicas x{world}"},
        "device_step": {"ms": 1000.0 * dev, "replaces_numpy_ms": 1000.0 * ref_steps,
                        "what": "edges + bend pairs + rest lengths + inverse masses (host arrays in and out)"},
        "gpu_launches": 33 * args.steps,  # kernels of one xpbd_gb300_prepare_cloth_device call
        "cpu_baseline": {"value": V / ref_full, "unit": "vertices/s", "cores": 1, "kind": "port",
                         "sample": "one numpy build of the same cloth"},
        "e2e": {"value": value, "unit": "vertices/s", "h2d_bytes_per_step": int(pos.nbytes + tris.nbytes + V),
                "d2h_bytes_per_step": int(3 * len(tris) * 12 + V * 4)},
    }
    print(json.dumps(line), flush=True)


def diff_measure(steps: int, warmup: int, torch) -> dict:
    """Differentiable form: one step = a 60-frame rollout of the 64 x 64 cloth
    and the adjoint of an L2 loss (vertex-substeps/s of the forward frames;
    the backward recomputes each frame once more)."""
    from xpbd_gb300.diff import DiffCloth

    sc = scene.diff_scene(64, 60)
    ks = torch.tensor(scene.compliance_field(len(sc.cloth.edges), 1e-7, 1.0, 0), device="cuda")
    kb = torch.tensor(scene.compliance_field(len(sc.cloth.bends), 1e-4, 1.0, 1), device="cuda")
    kts = torch.tensor(scene.compliance_field(len(sc.cloth.edges), 1e-7, 1.0, 2), device="cuda")
    ktb = torch.tensor(scene.compliance_field(len(sc.cloth.bends), 1e-4, 1.0, 3), device="cuda")
    dc = DiffCloth(sc.cloth, sc.options)
    target = dc.rollout(kts, ktb, sc.frames, sc.substeps, sc.iterations).clone()

    def step():
        x = dc.rollout(ks, kb, sc.frames, sc.substeps, sc.iterations)
        return dc.backward(2.0 * (x - target))

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        gs, gb = step()
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    t1 = time.perf_counter()
    for _ in range(steps):
        dc.rollout(ks, kb, sc.frames, sc.substeps, sc.iterations)
    torch.cuda.synchronize()
    fwd = time.perf_counter() - t1
    V = len(sc.cloth.positions_world)
    return {"value": V * sc.substeps * sc.frames * steps / el, "unit": METRIC, "ms_per_step": 1000.0 * el / steps,
            "forward_only": {"value": V * sc.substeps * sc.frames * steps / fwd, "unit": METRIC,
                             "ms_per_rollout": 1000.0 * fwd / steps},
            "grad_norms": {"stretch": float(gs.norm()), "bend": float(gb.norm())},
            "sizes": {"vertices": V, "edges": len(sc.cloth.edges), "bends": len(sc.cloth.bends), "frames": sc.frames,
                      "substeps": sc.substeps}}


def run_diff(args, world, rank, local):
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no differentiable rollout"}), flush=True)
        return
    import torch

    torch.cuda.set_device(local)
    from xpbd_gb300 import build

    build.build()
    d = diff_measure(args.steps, args.warmup, torch)
    value = d["value"] * world
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": d["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded compliance fields)",
        "config": {"workload": DESCRIPTIONS["diff"], **d["sizes"], "parallelism": f"replicas x{world}"},
        "forward_only": d["forward_only"], "grad_norms": d["grad_norms"],
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "inputs and gradients stay on the device (torch tensors)"},
    }
    print(json.dumps(line), flush=True)


def serve_measure(seconds: float, budget_gb: float, latency_ms: float | None, warmup: int, seed: int, torch,
                  clock_index: int | None = None) -> tuple[dict, dict | None]:
    """The request loop for `seconds` of Poisson arrivals (200/s); returns its
    statistics (results removed, their downloaded bytes kept) and the clock
    summary when sampled."""
    from xpbd_gb300.serving import ServingEngine

    reqs = scene.serving_requests(rate=200.0, duration=seconds, seed=seed)
    # warm-up: a few small requests through a separate engine (module load, first graph capture)
    warm = ServingEngine(hbm_budget_bytes=int(8e9))
    warm.run(scene.serving_requests(rate=50.0, duration=0.1, seed=99, v_range=(1000, 4000), horizon=(3, 5),
                                    max_requests=warmup), duration=None, drain=True)
    warm.close()
    torch.cuda.synchronize()
    eng = ServingEngine(hbm_budget_bytes=int(budget_gb * 1e9), frame_latency_ms=latency_ms)
    sampler = ClockSampler(clock_index) if clock_index is not None else None
    if sampler:
        sampler.__enter__()
    try:
        st = eng.run(reqs, duration=seconds)
        eng.close()  # waits for solvers still being built (their graph captures) before any device-wide sync
        torch.cuda.synchronize()
    finally:
        if sampler:
            sampler.__exit__(None, None, None)
    results = st.pop("results")
    st["offered_requests"] = len(reqs)
    st["d2h_bytes"] = int(sum(r.positions.nbytes for r in results))
    return st, (sampler.summary() if sampler else None)


def run_serving(args, world, rank, local):
    """Serving form: the request loop for --serve-seconds of Poisson
    arrivals; a "step" is one tick (every resident request advances one
    frame).  Each rank serves its own arrival stream (replicas)."""
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving loop; its CPU "
                              "restatement is timed by the batch256 / drop10k workloads"}), flush=True)
        return
    import torch

    torch.cuda.set_device(local)
    from xpbd_gb300 import build

    build.build()
    st, clocks = serve_measure(args.serve_seconds, args.serve_budget_gb, args.serve_latency_ms, args.warmup, rank,
                               torch, local)
    value = st["throughput"] * world
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": st["ticks"], "warmup": args.warmup,
        "ms_per_step": 1000.0 * st["elapsed_s"] / max(st["ticks"], 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded request stream)",
        "config": {"workload": DESCRIPTIONS["serve"], "seconds": args.serve_seconds, "offered_requests": st["offered_requests"],
                   "budget_gb": args.serve_budget_gb, "frame_latency_target_ms": args.serve_latency_ms,
                   "parallelism": f"replicas x{world}"},
        "serving": st,
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": st["d2h_bytes"] / max(st["ticks"], 1),
                "note": "the loop is end to end: requests enter from host arrays and results return to host memory"},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def time_plain_serial(native, scs, frames: int = 1) -> dict:
    """One ABI41 handle per cloth, each frame waited for before the next
    cloth steps: the order in which the reference add-on's handles run when
    every launch goes to one device stream (the reference launches its
    kernels on the legacy default stream, native/src/ssbl_xpbd_cuda_abi41.cu:
    4527, 6204 and most other launches)."""
    S, I = scs[0].substeps, scs[0].iterations
    V = sum(len(s.cloth.positions_world) for s in scs)
    total = 0.0
    for s in scs:
        solver = native.NativeXpbdSolver(s.cloth, s.options, s.static_triangles)
        solver.step(S, I, diagnostics=False, synchronize=True)
        t0 = time.perf_counter()
        for _ in range(frames):
            solver.step(S, I, diagnostics=False, synchronize=True)
        total += time.perf_counter() - t0
        solver.close()
    return {"value": V * S * frames / total, "unit": METRIC, "ms_per_step": 1000.0 * total / frames, "frames": frames,
            "handles": len(scs), "note": "handles stepped one after another, each frame synchronised"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batch256", choices=sorted(DESCRIPTIONS))
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--plain-frames", type=int, default=3, help="frames of the plain comparison (0 skips it)")
    ap.add_argument("--batch-cloths", type=int, default=256, help="cloths of the batch256 workload (smaller for profiling)")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-budget-gb", type=float, default=64.0)
    ap.add_argument("--serve-latency-ms", type=float, default=100.0,
                    help="frame-latency target of the serving admission (0: admission by memory only)")
    ap.add_argument("--autotune", type=int, default=1, help="1: launch configuration from the autotuner (default); 0: built-in defaults")
    ap.add_argument("--extras", type=int, default=1,
                    help="1: also measure plain32, drop10k, serving, diff and the reference solver (default line)")
    ap.add_argument("--profile-frame", action="store_true",
                    help="only: after the warm-up frames, one profiled frame (kernels serialised on the solver stream) "
                         "inside the NVTX range 'prof' (for ncu --nvtx-include), then its work counters as JSON")
    args = ap.parse_args()
    args.serve_latency_ms = args.serve_latency_ms if args.serve_latency_ms > 0 else None
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.workload == "serve":
        run_serving(args, world, rank, local)
        return
    if args.workload == "diff":
        run_diff(args, world, rank, local)
        return
    if args.workload == "prep":
        run_prep(args, world, rank, local)
        return
    if args.impl == "reference":
        # the reference arm builds its sample with the Python builders only
        # (no library of this repository is loaded)
        scene.set_native_prep(False)
        if args.workload == "batch256":
            scs = scene.batched_scenes(args.batch_cloths, seed=0, frames=120, only=sample_indices(args.batch_cloths))
        else:
            scs = workload(args.workload)
        run_reference(args, scs, world, rank)
        return
    scs = workload(args.workload, args.batch_cloths)
    if args.batch_cloths != 256 and args.workload == "batch256":
        nv = sum(len(s.cloth.positions_world) for s in scs)
        DESCRIPTIONS["batch256"] = DESCRIPTIONS["batch256"].replace("256 independent cloths", f"{args.batch_cloths} independent cloths").replace(
            "1,589,788 verts", f"{nv:,} verts")

    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from xpbd_gb300 import build, native

    build.build()
    V = sum(len(s.cloth.positions_world) for s in scs)
    E = sum(len(s.cloth.edges) for s in scs)
    T = sum(len(s.cloth.triangles) for s in scs)
    B = sum(len(s.cloth.bends) for s in scs)
    S, I = scs[0].substeps, scs[0].iterations
    batched = len(scs) > 1
    if batched:
        solver = native.NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs])
    else:
        solver = native.NativeXpbdSolver(scs[0].cloth, scs[0].options, scs[0].static_triangles)
    # launch configuration from the autotuner (cached per device and
    # workload; measured from the initial state, which it restores)
    tuned = solver.autotune(S, I, rounds=2) if args.autotune else None
    if args.profile_frame:
        for _ in range(args.warmup):
            solver.step(S, I, diagnostics=False, synchronize=True)
        torch.cuda.nvtx.range_push("prof")
        prof = solver.profile_frame(S, I)
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"workload": DESCRIPTIONS[args.workload], "launch_config": solver.launch_config(),
                          "counters": solver.profile_counters(),
                          "profile": {k: {"ms": ms, "launches": n} for k, (ms, n) in prof.items() if n}}))
        solver.close()
        return
    for _ in range(args.warmup):
        solver.step(S, I, diagnostics=False, synchronize=False)
    solver.synchronize()
    with ClockSampler(local) as clocks:
        total_ms = device_time(solver, S, I, args.steps, torch, world)
    launches_per_step = solver.last_step_launches()
    value = V * S * args.steps * world / (total_ms / 1000.0)

    # per-kernel profile of un-graphed frames (events around each launch on
    # the solver stream) and the work counters of the query kernels
    prof, counters = {}, {}
    reps = 2
    summed = ("ee_items", "ee_slots", "vt_items", "vt_slots", "ee_gathers")  # the others describe one build
    for _ in range(reps):
        p = solver.profile_frame(S, I)
        for k, (ms, n) in p.items():
            a = prof.setdefault(k, [0.0, 0])
            a[0] += ms
            a[1] += n
        for k, c in solver.profile_counters().items():
            counters[k] = counters.get(k, 0) + c if k in summed else c
    ranked = sorted(prof.items(), key=lambda kv: -kv[1][0])
    dominant = ranked[0][0]
    peak, peak_kind = peaks()
    roof = None
    # the dominant kind, or the largest one with a byte model
    for kind, (k_ms, k_n) in ranked:
        alg_total = algorithmic_bytes(kind, V, E, T, B, counters)
        avg_ms = k_ms / max(k_n, 1)
        if alg_total is None or avg_ms <= 0:
            continue
        # query counters cover all profiled frames: bytes per launch
        per_launch = alg_total / max(k_n, 1) if kind in ("edge_edge", "vertex_triangle") else alg_total
        achieved = per_launch / (avg_ms / 1000.0) / 1e9
        traffic = measured_traffic(kind, counters, k_n)
        roof = {"bound": "hbm", "kernel": kind, "dominant": kind == dominant, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_kind} (hbm_gbs)", "traffic": traffic,
                "traffic_source": ("ncu DRAM bytes (cold caches) per evaluated slot (edge-edge) or per insertion (edge hash) of one profiled frame on 64 cloths, "
                                   "scaled by this workload's units per launch" if traffic is not None else None),
                "avg_launch_us": avg_ms * 1000.0, "algorithmic_bytes_per_launch": per_launch,
                "byte_model": ("12 B per candidate gather (edge-edge: visited slots whose candidate id is above the query edge's)"
                               if kind in ("edge_edge", "vertex_triangle") else "per-kernel state bytes")}
        full = full_gather_bytes(kind, counters)
        if full is not None:
            full_launch = full / max(k_n, 1)
            roof["full_gather"] = {"bytes_per_launch": full_launch, "achieved": full_launch / (avg_ms / 1000.0) / 1e9,
                                   "frac": full_launch / (avg_ms / 1000.0) / 1e9 / peak,
                                   "model": "per item its rows and bucket range, per slot its id, per gather indices + rows"}
        break
    kernel_rooflines = {}
    for kind, (k_ms, k_n) in ranked:
        alg_total = algorithmic_bytes(kind, V, E, T, B, counters)
        if alg_total is None or k_n <= 0 or k_ms <= 0:
            continue
        per_launch = alg_total / k_n if kind in ("edge_edge", "vertex_triangle") else alg_total
        gbs = per_launch / (k_ms / k_n / 1000.0) / 1e9
        kernel_rooflines[kind] = {"achieved_gbs": gbs, "frac": gbs / peak, "ms_per_frame": k_ms / reps}
    profile_summary = {k: {"ms_per_frame": v[0] / reps, "launches_per_frame": v[1] / reps} for k, v in prof.items() if v[1]}

    # end to end through the C-ABI with host buffers: every frame the pin
    # targets of all cloths go up and all positions come back
    lib = native._load_library()
    out = torch.empty((V, 3), dtype=torch.float32).pin_memory().numpy()
    pin_idx, pin_pos, pin_w = [], [], []
    base = 0
    for s in scs:
        pin_idx.append(s.cloth.pin_indices.astype(np.int32) + base)
        pin_pos.append(s.cloth.pin_targets_world)
        pin_w.append(s.cloth.pin_weights)
        base += len(s.cloth.positions_world)
    pin_idx = torch.from_numpy(np.concatenate(pin_idx)).pin_memory().numpy()
    pin_pos = torch.from_numpy(np.ascontiguousarray(np.concatenate(pin_pos), np.float32)).pin_memory().numpy()
    pin_w = torch.from_numpy(np.ascontiguousarray(np.concatenate(pin_w), np.float32)).pin_memory().numpy()
    ip = pin_idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    pp = pin_pos.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    wp = pin_w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    h2d = pin_idx.nbytes + pin_pos.nbytes + pin_w.nbytes
    d2h = out.nbytes
    h = solver.handle
    fp = out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def e2e_frame():
        ok = lib.ssbl_update_pin_targets(h, ip, pp, wp, len(pin_idx)) and lib.ssbl_step_solver_ex(h, S, I, 0, 0) and \
            lib.ssbl_download_positions(h, fp, out.size)
        if not ok:
            raise RuntimeError(native._last_error(lib))

    # the same frames as the device-timed region: from the initial state,
    # W warm-up frames, then K timed frames
    if not lib.ssbl_reset_solver(h):
        raise RuntimeError(native._last_error(lib))
    for _ in range(args.warmup):
        e2e_frame()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_frame()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": V * S * args.steps * world / e2e_s, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000.0 * e2e_s / args.steps}
    assert np.isfinite(out).all()

    plain = time_plain(native, scs, args.plain_frames) if batched and args.plain_frames > 0 else None
    plain_serial = time_plain_serial(native, scs) if batched and args.plain_frames > 0 else None
    launch_cfg = solver.launch_config()
    solver.close()
    extras = {}
    if args.extras and rank == 0:
        extras["reference_gpu"] = time_reference_gpu(scs, max(args.plain_frames, 1), torch) if batched else None
        extras["plain32"] = time_single(native, torch, "plain32", 50, args.warmup)
        extras["drop10k"] = time_single(native, torch, "drop10k", 50, args.warmup)
        for name in ("plain32", "drop10k"):
            ref_single = time_reference_single(name, 20, args.warmup, torch)
            extras[f"reference_gpu_{name}"] = ref_single
            if "value" in ref_single:
                extras[f"{name}_over_reference"] = extras[name]["value"] / ref_single["value"]
        extras["diff"] = diff_measure(3, 1, torch)
        st, _ = serve_measure(args.serve_seconds, args.serve_budget_gb, args.serve_latency_ms, args.warmup, 0, torch)
        extras["serving"] = {"value": st["throughput"], "unit": METRIC, "workload": DESCRIPTIONS["serve"],
                             "seconds": args.serve_seconds, "frame_latency_target_ms": args.serve_latency_ms,
                             "frame_latency_ms_p50": st["frame_latency_ms_p50"],
                             "frame_latency_ms_p99": st["frame_latency_ms_p99"], "stats": st}

    if rank != 0:
        return
    cpu_value, cores, sample = cpu_oracle_rate(scs, args.cpu_budget)
    config = {"workload": DESCRIPTIONS[args.workload], "cloths": len(scs), "vertices": V, "edges": E, "triangles": T,
              "substeps": S, "iterations": I, "frames_per_step": 1,
              "l2": "256 MiB buffer written before every timed step", "parallelism": f"replicas x{world}"}
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded grid cloths, box/torus collider)", "config": config,
        "e2e": e2e, "gpu_launches": int(launches_per_step * args.steps), "clocks": clocks.summary(),
        "roofline": roof, "kernel_profile": profile_summary, "work_counters_per_frame": {k: (c / reps if k in summed else c) for k, c in counters.items()},
        "cpu_baseline": {"value": cpu_value, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample},
        "launch_config": {"config": launch_cfg, "autotune": tuned},
    }
    line["kernel_rooflines"] = kernel_rooflines
    if plain is not None:
        line["plain"] = plain
        line["batched_over_plain"] = value / plain["value"]
    if plain_serial is not None:
        line["plain_serial"] = plain_serial
        line["batched_over_plain_serial"] = value / plain_serial["value"]
    for k, v in extras.items():
        if v is not None:
            line[k] = v
    ref = extras.get("reference_gpu")
    if ref and "value" in ref:
        line["batched_over_reference_plain"] = value / ref["value"]
        line["e2e_over_reference_plain"] = e2e["value"] / ref["value"]
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
