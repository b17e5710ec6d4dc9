"""Builds libredgb.so (the CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

    python -m redgb.build          (from red.cuda.closeencounter_gb300/)

Each translation unit is compiled in parallel; the FP64-exact units get -fmad=false so
that no multiply-add is contracted (the reference builds with -fmad=false,
red.cuda/Makefile:17), and all host code gets -ffp-contract=off for the same reason.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)  # red.cuda.closeencounter_gb300
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG_DIR, "libredgb.so")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-Xcompiler", "-fvisibility=hidden", "-I", CSRC, "-I", INCLUDE]
# unit -> extra flags
UNITS = {
    "context.cu": ["-fmad=false"],
    "stages.cu": ["-fmad=false"],
    "gravity_fp64.cu": ["-fmad=false"],
    "gravity_mixed.cu": [],
    "ensemble.cu": ["-fmad=false"],
    "mlp.cu": [],
    "noalloc.cu": ["-fmad=false"],
    "ens_events.cu": ["-fmad=false"],
    "icgen.cu": ["-fmad=false"],
}


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libredgb.so")


def _sources():
    return [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "redgb.h"))
    files.append(os.path.join(INCLUDE, "redgb_types.h"))
    files.append(os.path.abspath(__file__))
    return files


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force=False, verbose=False, jobs=None):
    """Compile and link libredgb.so if any source changed.  Returns the library path."""
    if not force and not stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    units = _sources()

    def compile_one(u):
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        cmd = [exe, *ARCH, *COMMON, *UNITS[u], "-c", os.path.join(CSRC, u), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {u}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or len(units)) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
