"""Build of the native library ``formoniq_gb300/_lib/libformoniq_gb300.so``.

One nvcc per translation unit, in parallel, for sm_103a only; then one link.
The library is the product: the Python package binds it through ctypes and has
no other compute path.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libformoniq_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")] + ARCH


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the formoniq_gb300 CUDA library cannot be built")


def sources():
    """Translation units, the slowest compiles first (the 4D and 3D cell
    programs), so that the parallel build's makespan is not one late start."""
    def cost(f):
        return (0 if "_n4" in f else 1 if "_n3" in f else 2, f)

    return [os.path.join(CSRC, f) for f in sorted((f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp"))), key=cost)]


def _stale(src: str, obj: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "formoniq_gpu.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra=()) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if _stale(src, obj):
        cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr[-4000:]}")
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(_compile, srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs + ["-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
