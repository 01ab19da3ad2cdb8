"""Builds the mesoengine_gb300 CUDA library for sm_103a (in-tree, no cmake).

nvcc compiles each translation unit of csrc/ in parallel and links them into
mesoengine_gb300/_lib/libmeso_gb300.so; the C ABI is include/meso.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libmeso_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
# nvcc warnings are errors: a host-only call from device code (a "calling a
# __host__ function from a __host__ __device__ function" warning) compiles to
# undefined device code otherwise.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Werror", "all-warnings", "-Xcompiler",
         "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xcompiler", "-Wall,-Wno-unused-function",
         "-I", os.path.join(ROOT, "include")]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, obj, extra):
    cmd = [NVCC] + ARCH + FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    objs = []
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for s in srcs:
            o = os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o")
            objs.append(o)
            if force or _stale(o, [s] + hdrs):
                jobs.append(ex.submit(_compile, s, o, list(extra)))
        for j in jobs:
            j.result()
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".{os.getpid()}.tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
