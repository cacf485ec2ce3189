"""Builds liblsg.so (the CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

    python linear-solver_gb300/build.py            # incremental
    python linear-solver_gb300/build.py --force    # rebuild everything
    LSG_BOUNDS=1 python linear-solver_gb300/build.py   # bounds-checked debug build

The bounds-checked build (-DLSG_BOUNDS) checks every global and shared index
of the stencil marches, records the first one out of range and skips the
access (lsg_bounds_errors reads it): the substitute for a sanitizer run.

Each translation unit is compiled in parallel into ``_build/`` and linked
into ``liblsg.so`` next to this file.  No CMake, no torch extension machinery:
the library is plain C ABI and loads with ctypes from any language.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BOUNDS = os.environ.get("LSG_BOUNDS", "") == "1"
BUILD = os.path.join(HERE, "_build_bounds" if BOUNDS else "_build")
LIB = os.path.join(HERE, "liblsg.so")
VARIANT = os.path.join(HERE, "_build", "liblsg.variant")  # which build the library holds

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-ffp-contract=off",  # host arithmetic identical on x86 and Arm
              "-diag-suppress", "177", f"-I{os.path.join(ROOT, 'include')}"] + (["-DLSG_BOUNDS"] if BOUNDS else [])
SOURCES = ["lsg_kernels_f64.cu", "lsg_kernels_f32.cu", "lsg_kernels_c128.cu", "lsg_kernels_c64.cu",
           "lsg_batch_f64.cu", "lsg_batch_f32.cu", "lsg_batch_c128.cu", "lsg_batch_c64.cu",
           "lsg_small.cu", "lsg_solvers.cu", "lsg_batch.cu", "lsg_tune.cu", "lsg_krylov.cu", "lsg_csr.cu", "lsg_icc.cu", "lsg_dot.cu", "lsg_compat.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc)]
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if force or _stale(obj, [path] + _headers()):
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-c", path, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [_nvcc(), "-x", "cu", *ARCH, *NVCC_FLAGS, "-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), SOURCES))
    variant = "bounds" if BOUNDS else "normal"
    held = open(VARIANT).read().strip() if os.path.exists(VARIANT) else ""
    if force or held != variant or _stale(LIB, objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.makedirs(os.path.dirname(VARIANT), exist_ok=True)
        with open(VARIANT, "w") as f:
            f.write(variant)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
