#!/usr/bin/env python3
"""Benchmark of the GB300 XPBD cloth step (vertex-substeps/s).

Workload (default ``drop10k``): a 100 x 100 cloth (10,000 vertices, 19,602
triangles) with seeded +-1 mm jitter dropped onto a sphere (r = 0.3 m) and a
64^3 static SDF of a box and a torus, strict spatial-hash self collision with
2 mm thickness, friction 0.3; 10 substeps x 2 iterations per frame.  A
"step" is one frame.  Inputs are seeded synthetic (no dataset exists).

Timing: W untimed warm-up frames, then K frames, each bracketed by CUDA
events on the solver's own stream; before every timed frame a 256 MiB buffer
is written on that stream so L2 (129 MB) starts cold (the cloth's state is
far smaller than L2).  ``value`` = vertices x substeps x K x N / time.

Also reported: ``e2e`` through the C-ABI with host buffers (frame inputs
uploaded, positions downloaded every frame), the per-kernel profile and the
roofline of the dominant kernel, SM clocks sampled during the timed region,
and the CPU oracle timed on a bounded sample of the same workload.

``--impl reference``: the reference's step has no CPU implementation and its
CUDA solver cannot be carried to the GPU machine, so that arm times the CPU
restatement of the reference's algorithm (oracle/) with all host threads.
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

# Compulsory bytes per launch of each kernel kind: state rows read and
# written once (16-byte rows, 4-byte scalars), constraint streams read once.
# Candidate gathers of the self-collision queries are not counted, so these
# are lower bounds for those kinds.
def kernel_bytes(kind: str, V: int, E: int, T: int) -> float | None:
    table = {
        "predict": V * (16 * 2 + 16 * 3 + 4),        # R pos vel, W pos prev vel, R pin weight
        "stretch_pass": V * (16 * 3 * 2 + 4 + 4 + 4) + 2 * E * 8,  # R/W pos prev vel, pin, inv, CSR off; 2E entries
        "vertex_pass": V * (16 * 3 * 2 + 4 + 4),
        "neighbors": V * (16 + 16 + 4) + V * 4,        # pos, cell, count
        "vertex_vertex": V * (4 + 16 + 16 + 4 + 32),   # count, pos, prev, inv, acc
        "vertex_triangle": V * (16 + 8),               # pos, bucket range
        "edge_edge": E * (8 + 32 + 8),                 # edge, endpoints, bucket range
        "self_apply": V * (32 * 2 + 16 * 2 * 2 + 4),   # acc R/W, pos prev R/W, inv
    }
    return table.get(kind)


def workload(name: str):
    if name == "drop10k":
        return scene.drop_scene(100, 200, seed=0, self_mode=2)
    if name == "plain32":
        return scene.plain_grid_scene(32, 120)
    raise SystemExit(f"unknown workload {name}")


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


def cpu_oracle_rate(sc, budget_s: float, warm: int = 1) -> tuple[float, int, str]:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import xpbd_oracle

    threads = xpbd_oracle.set_threads(os.cpu_count() or 1)
    o = xpbd_oracle.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    for _ in range(warm):
        o.step(sc.substeps, sc.iterations)
    frames, t0 = 0, time.perf_counter()
    while True:
        o.step(sc.substeps, sc.iterations)
        frames += 1
        el = time.perf_counter() - t0
        if el >= budget_s or frames >= 400:
            break
    V = len(sc.cloth.positions_world)
    return V * sc.substeps * frames / el, threads, f"{frames} frames after {warm} warm-up, {el:.1f} s"


def run_reference(args, sc, world, rank):
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import xpbd_oracle

    threads = xpbd_oracle.set_threads(os.cpu_count() or 1)
    o = xpbd_oracle.OracleSolver.from_scene(sc.cloth, sc.options, sc.static_triangles)
    for _ in range(args.warmup):
        o.step(sc.substeps, sc.iterations)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(sc.substeps, sc.iterations)
    el = time.perf_counter() - t0
    V = len(sc.cloth.positions_world)
    value = V * sc.substeps * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": args.workload_desc, "vertices": V, "substeps": sc.substeps, "iterations": sc.iterations},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} frames of the same workload after {args.warmup} warm-up frames"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's step exists only as CUDA code; this arm is the C restatement of its algorithm on the host cores",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="drop10k", choices=["drop10k", "plain32"])
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    sc = workload(args.workload)
    args.workload_desc = {
        "drop10k": "10k cloth (100x100 grid, 19,602 tris) dropped on a sphere + 64^3 box/torus SDF, strict self "
                   "collision 2 mm, friction 0.3, 10 substeps x 2 iterations per frame",
        "plain32": "plain 32x32 grid (1,024 verts), two pinned corners, ground, 10 substeps x 2 iterations",
    }[args.workload]
    if args.impl == "reference":
        run_reference(args, sc, world, rank)
        return

    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from xpbd_gb300 import build, native

    build.build()
    V = len(sc.cloth.positions_world)
    E = len(sc.cloth.edges)
    T = len(sc.cloth.triangles)
    S, I = sc.substeps, sc.iterations
    solver = native.NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    for _ in range(args.warmup):
        solver.step(S, I, diagnostics=False, synchronize=False)
    solver.synchronize()
    stream = torch.cuda.ExternalStream(solver.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
            events[k][0].record(stream)
            solver.step(S, I, diagnostics=False, synchronize=False)
            events[k][1].record(stream)
        torch.cuda.synchronize()
    total_ms = sum(a.elapsed_time(b) for a, b in events)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        torch.distributed.barrier()
    launches_per_step = solver.last_step_launches()
    value = V * S * args.steps * world / (total_ms / 1000.0)

    # per-kernel profile of one un-graphed frame (events around each launch)
    prof = {}
    for _ in range(3):
        p = solver.profile_frame(S, I)
        for k, (ms, n) in p.items():
            a = prof.setdefault(k, [0.0, 0])
            a[0] += ms
            a[1] += n
    dominant = max(prof.items(), key=lambda kv: kv[1][0])[0]
    dom_ms, dom_n = prof[dominant]
    avg_ms = dom_ms / max(dom_n, 1)
    peak, peak_kind = peaks()
    alg = kernel_bytes(dominant, V, E, T)
    roof = None
    if alg is not None and avg_ms > 0:
        achieved = alg / (avg_ms / 1000.0) / 1e9
        roof = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} (hbm_gbs)", "traffic": None,
                "avg_launch_us": avg_ms * 1000.0, "algorithmic_bytes_per_launch": alg}
    profile_summary = {k: {"ms_per_frame": v[0] / 3.0, "launches_per_frame": v[1] / 3.0} for k, v in prof.items() if v[1]}

    # end to end through the C-ABI with host buffers
    lib = native._load_library()
    out = torch.empty((V, 3), dtype=torch.float32).pin_memory().numpy()
    colliders = native.colliders_from_options(sc.options)
    fi = native.NativeFrameInputs()
    fi.update_runtime_colliders = 1
    fi.runtime_colliders = colliders
    h2d = ctypes.sizeof(native.NativeRuntimeColliders)
    d2h = out.nbytes
    h = solver.handle
    fp = out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    for _ in range(2):
        lib.ssbl_update_frame_inputs(h, ctypes.byref(fi))
        lib.ssbl_step_solver_ex(h, S, I, 0, 0)
        lib.ssbl_download_positions(h, fp, out.size)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ok = lib.ssbl_update_frame_inputs(h, ctypes.byref(fi)) and lib.ssbl_step_solver_ex(h, S, I, 0, 0) and \
            lib.ssbl_download_positions(h, fp, out.size)
        if not ok:
            raise RuntimeError(native._last_error(lib))
    e2e_s = time.perf_counter() - t0
    e2e = {"value": V * S * args.steps * world / e2e_s, "unit": METRIC, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": 1000.0 * e2e_s / args.steps}
    assert np.isfinite(out).all()

    if rank != 0:
        return
    cpu_value, cores, sample = cpu_oracle_rate(sc, args.cpu_budget)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded grid cloth, box/torus collider)",
        "config": {"workload": args.workload_desc, "vertices": V, "edges": E, "triangles": T, "substeps": S,
                   "iterations": I, "frames_per_step": 1, "l2": "256 MiB buffer written before every timed step",
                   "parallelism": f"replicas x{world}"},
        "e2e": e2e, "gpu_launches": int(launches_per_step * args.steps), "clocks": clocks.summary(),
        "roofline": roof, "kernel_profile": profile_summary,
        "cpu_baseline": {"value": cpu_value, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
