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
RECO = os.path.join(PKG, "epet_reco")  # C++ driver over the drop-in header
SOURCES = ["runtime.cu", "geometry.cu", "workqueue.cu", "sm_build.cu", "sort.cu",
           "spmv.cu", "mlem.cu", "compat.cu", "compress.cu", "tune.cu", "batch.cu",
           "grouped.cu", "hdf5_io.cpp"]
HEADERS = ["common.cuh", "internal.h", "spmv.cuh", "rows.cuh", "mlem_internal.h"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def cuda_libdir() -> str:
    base = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    for d in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"),
              os.path.join("targets", "x86_64-linux", "lib")):
        if os.path.exists(os.path.join(base, d, "libcudart.so")):
            return os.path.join(base, d)
    return os.path.join(base, "lib64")


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


def _torch_flags():
    import sysconfig

    import torch
    tdir = os.path.dirname(torch.__file__)
    inc = [os.path.join(tdir, "include"), os.path.join(tdir, "include", "torch", "csrc", "api",
                                                       "include"),
           sysconfig.get_paths()["include"], os.path.join(ROOT, "include"),
           os.path.join(os.path.dirname(cuda_libdir()), "include")]
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    cflags = ["-O2", "-std=c++17", "-fPIC", f"-D_GLIBCXX_USE_CXX11_ABI={abi}",
              "-DTORCH_EXTENSION_NAME=_autograd", "-DTORCH_API_INCLUDE_EXTENSION_H",
              "-Wno-deprecated-declarations"] + ["-I" + d for d in inc]
    libdir = os.path.join(tdir, "lib")
    ldflags = ["-L" + libdir, "-lc10", "-lc10_cuda", "-ltorch", "-ltorch_cpu", "-ltorch_cuda",
               "-ltorch_python", "-L" + PKG, "-lepet_gb300", "-L" + cuda_libdir(), "-lcudart",
               "-Wl,-rpath," + libdir, "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + cuda_libdir()]
    return cflags, ldflags


def autograd_path() -> str:
    import sysconfig
    return os.path.join(PKG, "_autograd" + sysconfig.get_config_var("EXT_SUFFIX"))


def _compile_autograd() -> str:
    src = os.path.join(CSRC, "autograd.cpp")
    obj = os.path.join(BUILD, "autograd.o")
    deps = [src, os.path.join(ROOT, "include", "epet_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(map(os.path.getmtime, deps)):
        return obj
    cflags, _ = _torch_flags()
    r = subprocess.run(["g++"] + cflags + ["-c", src, "-o", obj], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"autograd extension compile failed:\n{r.stderr[-4000:]}")
    return obj


def _link_autograd(obj: str) -> None:
    out = autograd_path()
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(obj),
                                                           os.path.getmtime(LIB)):
        return
    _, ldflags = _torch_flags()
    r = subprocess.run(["g++", "-shared", obj, "-o", out] + ldflags, capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"autograd extension link failed:\n{r.stderr[-4000:]}")


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        ag = ex.submit(_compile_autograd)
        objs = list(ex.map(_compile, SOURCES))
        ag_obj = ag.result()
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(map(os.path.getmtime, objs)):
        # shared CUDA runtime: in a process that already loaded one (torch),
        # the loader reuses it, so there is a single runtime instance
        cmd = [nvcc(), "-shared", "-cudart", "shared", "-gencode",
               "arch=compute_103a,code=sm_103a", "-o", LIB] + objs + \
            ["-Xlinker", "-rpath=" + cuda_libdir()]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    _build_driver()
    _link_autograd(ag_obj)
    if verbose:
        print(LIB)
    return LIB


def _build_driver() -> None:
    src = os.path.join(CSRC, "reco_main.cpp")
    deps = [src, LIB, os.path.join(ROOT, "include", "epet_gb300_shim.hpp")]
    if os.path.exists(RECO) and os.path.getmtime(RECO) >= max(map(os.path.getmtime, deps)):
        return
    cmd = [nvcc(), "-O2", "-std=c++17", "-x", "cu", "-cudart", "shared", "-gencode",
           "arch=compute_103a,code=sm_103a", "-I" + os.path.join(ROOT, "include"), src,
           "-o", RECO, "-L" + PKG, "-lepet_gb300", "-Xlinker", "-rpath=$ORIGIN",
           "-Xlinker", "-rpath=" + cuda_libdir()]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stderr}")


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
