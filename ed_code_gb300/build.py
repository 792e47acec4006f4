"""Build the CUDA library libedgpu.so (sm_103a) in-tree.

Each translation unit under csrc/ is compiled by its own nvcc process (in
parallel), then linked into ed_code_gb300/libedgpu.so.  The C++ adapter that
re-exports the reference's C++ signatures is built into libedgpu_ref.so on
top of it.  Nothing is installed outside the package directory.

usage: python -m ed_code_gb300.build [--verbose] [--ptxas-info]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libedgpu.so")
REF_LIB = os.path.join(HERE, "libedgpu_ref.so")

CUDA_UNITS = ["capi.cu", "basis.cu", "hv.cu", "lanczos.cu", "lanczos_mixed.cu", "targets.cu", "hv_noalloc.cu",
              "batch.cu", "tridiag_dev.cu", "dense.cu",
              "hv_block.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "edgpu.h"))
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", os.path.join(ROOT, "include")]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]
    objs = []
    jobs = []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or ptxas_info or _stale(obj, [src] + headers):
            jobs.append([nvcc()] + flags + ["-c", src, "-o", obj])
    out = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            out = list(ex.map(lambda c: _run(c, verbose), jobs))
    if ptxas_info:
        for o in out:
            sys.stdout.write(o)
    if force or _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"], verbose)
    adapter = os.path.join(CSRC, "ref_adapter.cpp")
    if os.path.exists(adapter) and (force or _stale(REF_LIB, [adapter, LIB] + headers)):
        _run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-o", REF_LIB,
              adapter, "-L", HERE, "-ledgpu", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    build(verbose="--verbose" in sys.argv, ptxas_info="--ptxas-info" in sys.argv, force="--force" in sys.argv)
    print(LIB)
