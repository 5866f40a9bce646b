"""Launch-configuration autotuner front end and its cache.

The search itself runs in the library (xpbd_gb300_autotune): coordinate
descent over the block sizes of each kernel class and the tile choices
(lanes per primitive of the hash build, lanes per item of the strict group
queries), each candidate timed as the fastest of a few profiled frames from
the same saved state.  No choice changes a result, so tuning is safe to run
on a live solver; its state is restored afterwards.

The chosen configuration is cached in a JSON file keyed by the device, the
library build and a workload signature (cloth, vertex, edge and triangle
counts, the self-collision mode mix, dynamic and SDF colliders, substeps and
iterations), so a workload seen before starts with its configuration
without measuring again.  The cache lives at $XPBD_GB300_TUNE_CACHE, else
~/.cache/xpbd_gb300/launch_tune.json.
"""
from __future__ import annotations

import hashlib
import json
import os
import time


def cache_path() -> str:
    p = os.environ.get("XPBD_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "xpbd_gb300", "launch_tune.json")


def device_name() -> str:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        pass
    return "cuda"


def library_id(lib_path: str | None) -> str:
    """Size and modification time of the loaded library (a rebuild may change
    the kernels, so its tuning starts over)."""
    if not lib_path or not os.path.exists(lib_path):
        return "unknown"
    st = os.stat(lib_path)
    return f"{st.st_size}-{int(st.st_mtime)}"


def workload_key(info: dict, substeps: int, iterations: int, device: str, lib: str) -> str:
    body = {"device": device, "library": lib, "substeps": int(substeps), "iterations": int(iterations),
            **{k: int(v) for k, v in sorted(info.items())}}
    return hashlib.sha1(json.dumps(body, sort_keys=True).encode()).hexdigest()


def load_cache(path: str) -> dict:
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store(path: str, key: str, entry: dict) -> None:
    data = load_cache(path)
    data[key] = entry
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(solver, substeps: int, iterations: int, rounds: int = 2, use_cache: bool = True, path: str | None = None) -> dict:
    """Apply the cached configuration for this workload, or measure one and
    cache it.  Returns {"config", "cached", "tuned_ms", "default_ms",
    "seconds"}."""
    path = path or cache_path()
    lib_path = getattr(getattr(solver, "_lib", None), "_name", None)
    key = workload_key(solver.solver_info(), substeps, iterations, device_name(), library_id(lib_path))
    if use_cache:
        hit = load_cache(path).get(key)
        if isinstance(hit, dict) and isinstance(hit.get("config"), dict):
            solver.set_launch_config(hit["config"])
            return {**hit, "cached": True, "seconds": 0.0}
    t0 = time.perf_counter()
    tuned_ms, default_ms = solver._autotune_native(substeps, iterations, rounds)
    entry = {"config": solver.launch_config(), "tuned_ms": tuned_ms, "default_ms": default_ms}
    if use_cache:
        try:
            store(path, key, entry)
        except OSError:
            pass  # a read-only home directory keeps the tuning for this process only
    return {**entry, "cached": False, "seconds": time.perf_counter() - t0}
