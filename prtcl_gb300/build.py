"""Build the CUDA library in-tree: prtcl_gb300/libprtcl_gpu.so (sm_103a).

Each translation unit is compiled in parallel with
    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -fmad=false
(no fused multiply-add: the FP32 procedures reproduce the reference's
scalar arithmetic bit for bit) and linked with the static CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libprtcl_gpu.so")
SOURCES = ["model.cu", "nhood.cu", "schemes.cu", "capi.cu", "noalloc.cu", "batch.cu", "server.cu", "archive.cu",
           "vtk.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "prtcl_gpu.h"), os.path.join(HERE, "..", "include", "prtcl_gpu.hpp"),
        os.path.join(HERE, "host", "prtcl_gpu_run.cpp"), __file__]


def up_to_date():
    if not os.path.exists(LIB) or not os.path.exists(os.path.join(HERE, "bin", "prtcl_gpu_run")):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OBJ, src.replace(".cu", ".o"))
        # the sweep kernels' variants make schemes.cu the longest unit:
        # its device code is optimised in parallel partitions
        split = [f"--split-compile={min(8, os.cpu_count() or 1)}"] if src == "schemes.cu" else []
        cmd = [cc, *ARCH, *FLAGS, *split, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver()
    return LIB


DRIVER_SRC = os.path.join(HERE, "host", "prtcl_gpu_run.cpp")
DRIVER = os.path.join(HERE, "bin", "prtcl_gpu_run")


def build_driver():
    """The native driver (host C++ over the C++ facade), linked against the
    library with an rpath to it."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for the native driver")
    os.makedirs(os.path.dirname(DRIVER), exist_ok=True)
    cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(HERE, "..", "include"), DRIVER_SRC,
           "-L", HERE, "-lprtcl_gpu", "-Wl,-rpath,$ORIGIN/..", "-o", DRIVER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build(force=True, verbose=v or bool(extra), extra=extra))
