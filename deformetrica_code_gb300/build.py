"""Builds libgbkernel.so (the sm_103a CUDA kernels and their C ABI) in-tree.

Every ``csrc/*.cu`` file is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
``deformetrica_code_gb300/libgbkernel.so`` (with cuFFT for the particle-mesh kernel). Rebuilds only
when a source is newer than the library. No CMake, no torch extension machinery: the library is
plain C ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbkernel.so")
# the bounds-checked build (-DGBK_BOUNDS_CHECK=1: every target / source index of the kernel sums
# checked, a failure reported as GBK_ERR_BOUNDS by gbk_synchronize); for tests, not the default
CHECKED_BUILD_DIR = os.path.join(HERE, "_build_checked")
CHECKED_LIB = os.path.join(HERE, "libgbkernel_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbkernel.so")


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps() -> list[str]:
    return (sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def up_to_date(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force: bool = False, verbose: bool = False, jobs: int | None = None, bounds_check: bool = False) -> str:
    """Builds libgbkernel.so, or with bounds_check=True libgbkernel_checked.so; returns its path."""
    LIB = CHECKED_LIB if bounds_check else globals()["LIB"]
    BUILD_DIR = CHECKED_BUILD_DIR if bounds_check else globals()["BUILD_DIR"]
    flags = NVCC_FLAGS + (["-DGBK_BOUNDS_CHECK=1"] if bounds_check else [])
    if not force and up_to_date(LIB):
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = sources()
    newest_header = max(os.path.getmtime(p) for p in _deps())

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest_header
                and os.path.getmtime(obj) >= os.path.getmtime(src)):
            return obj
        cmd = [nvcc, *ARCH, *flags, "-c", src, "-o", obj + ".tmp"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{res.stderr[-4000:]}")
        if verbose and res.stderr:
            print(res.stderr)
        os.replace(obj + ".tmp", obj)
        return obj

    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    # cuFFT (the particle-mesh kernel) from the toolkit this nvcc belongs to, found at run time by rpath
    cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcufft", "-Xlinker", "-rpath", "-Xlinker", cudalib]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, bounds_check="--bounds-check" in sys.argv[1:]))
