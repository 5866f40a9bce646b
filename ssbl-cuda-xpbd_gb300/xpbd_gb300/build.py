"""Build recipe of the GB300 XPBD shared library.

Compiles the CUDA sources under ``csrc/`` for sm_103a with nvcc (one
``-gencode``, translation units in parallel) and links
``lib/libssbl_xpbd_cuda_abi41.so``.  The basename keeps ``abi41`` because the
reference's bridge enables indexed dynamic triangles only for such a library
(native_backend.py:905-906).

Numerics flags: ``-fmad=false`` plus IEEE division and square root, so every
kernel performs exactly the single-precision operations written in the source
(explicit ``fmaf`` where the reference fuses), which is what lets the CPU
oracle reproduce results bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_NAME = "libssbl_xpbd_cuda_abi41.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-ftz=false",
    "-Xcompiler",
    "-fPIC,-fvisibility=hidden,-ffp-contract=off",
    "-I" + os.path.join(REPO_ROOT, "include"),
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the GB300 XPBD library needs the CUDA toolkit to build")
    return path


def library_path() -> str:
    return os.path.join(LIB_DIR, LIB_NAME)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(REPO_ROOT, "include")
    hdrs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hdrs


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile (when sources changed) and return the library path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    exe = nvcc()
    headers = _headers()
    sources = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    objects = []
    jobs = []
    for src in sources:
        src_path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objects.append(obj)
        if force or _stale(obj, [src_path] + headers):
            jobs.append([exe, *ARCH, *NVCC_FLAGS, "-c", src_path, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{proc.stdout}\n{proc.stderr}")
        if verbose and proc.stderr.strip():
            print(proc.stderr, file=sys.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as pool:
        list(pool.map(run, jobs))
    lib = library_path()
    if force or jobs or _stale(lib, objects):
        run([exe, *ARCH, "-shared", "-o", lib, *objects, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
