"""Build recipe of the reference's own CUDA solver (test infrastructure).

The reference solver (native/src/ssbl_xpbd_cuda_abi41.cu) is compiled from
its own sources, unchanged, with the flags of its own build
(native/CMakeLists.txt:55,109 and the Release configuration of
native/build_abi41.ps1: --use_fast_math, separable compilation, static CUDA
runtime, -O3), retargeted from sm_89 to sm_103a.  It serves two purposes
only: the GPU comparator of the parity tests and the reference timing beside
the benchmark.  Nothing in the product links or loads it.

Two steps, because the machine that has the reference checkout is not the
machine that has the GPU (an aarch64 host that runs no binary built here):

  python oracle/build_ref.py bundle --ref-root DIR
      packs the four reference files the build needs into
      oracle/_ref/reference_src.tar.gz (git-ignored, never committed) so the
      GPU machine can compile them;
  python oracle/build_ref.py build [--ref-root DIR]
      compiles, from DIR when it holds the reference, else from the bundle
      unpacked into oracle/_ref/src:
        oracle/_ref/libssbl_xpbd_cuda_abi41_ref.so  the reference solver with
            the probe of oracle/ref_probe.cu in the same translation unit
            (read access to its hash tables and neighbour lists);
        oracle/_ref/abi41_smoke_ref      the reference's known-answer program
            (native/smoke/abi41_smoke.cpp) linked to the reference solver;
        oracle/_ref/abi41_smoke_product  the same program, unchanged, linked
            to this repository's library.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tarfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BUNDLE = os.path.join(REF_DIR, "reference_src.tar.gz")
UNPACKED = os.path.join(REF_DIR, "src")
REPO = os.path.dirname(HERE)
PRODUCT_LIB_DIR = os.path.join(REPO, "ssbl-cuda-xpbd_gb300", "lib")
REF_LIB = os.path.join(REF_DIR, "libssbl_xpbd_cuda_abi41_ref.so")
SMOKE_REF = os.path.join(REF_DIR, "abi41_smoke_ref")
SMOKE_PRODUCT = os.path.join(REF_DIR, "abi41_smoke_product")

FILES = [
    "native/include/ssbl_xpbd_cuda.h",
    "native/include/ssbl_abi41_cuda_types.cuh",
    "native/src/ssbl_xpbd_cuda_abi41.cu",
    "native/smoke/abi41_smoke.cpp",
]

# native/CMakeLists.txt: CUDA_SEPARABLE_COMPILATION ON, CUDA_RUNTIME_LIBRARY
# Static, --use_fast_math; Release adds -O3 -DNDEBUG.
REF_NVCC_FLAGS = ["--use_fast_math", "-rdc=true", "-O3", "-DNDEBUG", "-std=c++17", "-cudart", "static"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _has_sources(root: str) -> bool:
    return bool(root) and all(os.path.isfile(os.path.join(root, f)) for f in FILES)


def bundle(ref_root: str) -> str:
    if not _has_sources(ref_root):
        raise SystemExit(f"reference sources not found under {ref_root}")
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = BUNDLE + ".tmp"
    with tarfile.open(tmp, "w:gz") as tar:
        for f in FILES:
            tar.add(os.path.join(ref_root, f), arcname=f)
    os.replace(tmp, BUNDLE)
    return BUNDLE


def source_root(ref_root: str | None) -> str:
    if ref_root and _has_sources(ref_root):
        return ref_root
    if not os.path.isfile(BUNDLE):
        raise SystemExit("no reference sources: neither a reference checkout nor oracle/_ref/reference_src.tar.gz")
    if not _has_sources(UNPACKED) or os.path.getmtime(BUNDLE) > os.path.getmtime(os.path.join(UNPACKED, FILES[2])):
        shutil.rmtree(UNPACKED, ignore_errors=True)
        os.makedirs(UNPACKED)
        with tarfile.open(BUNDLE, "r:gz") as tar:
            for member in tar.getmembers():
                if member.name not in FILES:
                    raise SystemExit(f"unexpected member {member.name} in the reference bundle")
            tar.extractall(UNPACKED)
    return UNPACKED


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"failed: {' '.join(cmd)}\n{proc.stdout[-2000:]}\n{proc.stderr[-4000:]}")


def build(ref_root: str | None, product: bool = True) -> list[str]:
    root = source_root(ref_root)
    os.makedirs(REF_DIR, exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(root, "native", "include")
    cu = os.path.join(root, "native", "src", "ssbl_xpbd_cuda_abi41.cu")
    smoke = os.path.join(root, "native", "smoke", "abi41_smoke.cpp")
    probe = os.path.join(HERE, "ref_probe.cu")
    built = []

    def lib_job():
        if _stale(REF_LIB, [cu, probe]):
            _run([nvcc, *ARCH, *REF_NVCC_FLAGS, "-shared", "-Xcompiler", "-fPIC", "-Xlinker", "--exclude-libs,ALL",
                  "-I" + inc, f'-DREF_ABI41_SOURCE="{cu}"', "-o", REF_LIB, probe])
        return REF_LIB

    def smoke_job(target: str, lib_dir: str, lib_name: str, dep: str):
        if _stale(target, [smoke, dep]):
            _run(["g++", "-std=c++17", "-O2", "-Wall", "-I" + inc, smoke, "-o", target, "-L" + lib_dir,
                  "-l" + lib_name, "-Wl,-rpath," + lib_dir])
        return target

    with ThreadPoolExecutor(max_workers=2) as pool:
        lib_future = pool.submit(lib_job)
        product_lib = os.path.join(PRODUCT_LIB_DIR, "libssbl_xpbd_cuda_abi41.so")
        prod_future = None
        if product and os.path.exists(product_lib):
            prod_future = pool.submit(smoke_job, SMOKE_PRODUCT, PRODUCT_LIB_DIR, "ssbl_xpbd_cuda_abi41", product_lib)
        built.append(lib_future.result())
        built.append(smoke_job(SMOKE_REF, REF_DIR, "ssbl_xpbd_cuda_abi41_ref", REF_LIB))
        if prod_future is not None:
            built.append(prod_future.result())
    return built


def main(argv: list[str]) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("step", choices=["bundle", "build"])
    ap.add_argument("--ref-root", default=os.environ.get("SSBL_REFERENCE_ROOT"))
    args = ap.parse_args(argv)
    if args.step == "bundle":
        print(bundle(args.ref_root))
    else:
        for path in build(args.ref_root):
            print(path)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
