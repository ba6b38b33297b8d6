"""Build libmlff_gb300.so (sm_103a) in-tree with nvcc.

Every translation unit under csrc/ is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
mlff-distiller_gb300/_build/libmlff_gb300.so (static CUDA runtime).  No
fast-math: the radius-graph decision relies on IEEE-rounded float32.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PROJECT = os.path.dirname(HERE)
CSRC = os.path.join(PROJECT, "csrc")
BUILD = os.path.join(PROJECT, "_build")
REPO = os.path.dirname(PROJECT)
INCLUDE = os.path.join(REPO, "include")
LIB_NAME = "libmlff_gb300.so"
LIB_PATH = os.path.join(BUILD, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmlff_gb300.so")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                  + glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers())


def build(verbose: bool = False, force: bool = False, extra_flags=None) -> str:
    """Compile and link; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    flags = NVCC_FLAGS + list(extra_flags or [])
    srcs = _sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    jobs = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, s)]

    def compile_one(so):
        s, o = so
        cmd = [nv, *ARCH, *flags, "-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(s)}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return o

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4) or 1) as ex:
        list(ex.map(compile_one, jobs))
    if jobs or not os.path.exists(LIB_PATH):
        tmp = LIB_PATH + ".tmp"
        cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
