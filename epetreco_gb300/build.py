"""Builds the CUDA library ``libepet_gb300.so`` in-tree with nvcc.

One ``-gencode`` (sm_103a), translation units compiled in parallel, host
code without floating-point contraction (the geometry's float sequence must
round like the reference's host build on both x86_64 and aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libepet_gb300.so")
SOURCES = ["runtime.cu", "geometry.cu", "workqueue.cu", "sm_build.cu", "sort.cu",
           "spmv.cu", "mlem.cu"]
HEADERS = ["common.cuh", "internal.h", "spmv.cuh"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


FLAGS = ["-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-Wall",
         "-I" + os.path.join(ROOT, "include")]


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, src + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
        [os.path.join(ROOT, "include", "epet_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(map(os.path.getmtime, deps)):
        return obj
    cmd = [nvcc()] + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(map(os.path.getmtime, objs)):
        cmd = [nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB] + \
            objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
