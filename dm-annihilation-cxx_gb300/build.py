"""Builds the in-tree native libraries for sm_103a (GB300).

    libdmann.so   CUDA kernels + the C ABI of include/dmann.h
    libannmap.so  the C++ host API (Parameters / DataReader / MapGenerator)
                  layered on the C ABI

Translation units compiled with -fmad=false are those whose FP64 arithmetic
must round exactly like the CPU map path (per-particle geometry, the plain
FP64 form).  Objects are compiled in parallel; a unit is rebuilt only when
it or a header changed.  Usage: ``python build.py [--force]``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(REPO, "include")]

# (source, fmad)
CUDA_UNITS = [("prep.cu", False), ("disc_plain.cu", False), ("disc_comp.cu", True), ("disc_seg.cu", True),
              ("capi.cu", True), ("noalloc.cu", True), ("adjoint.cu", False),
              ("peaks.cu", True), ("halocore.cu", False)]
CXX_UNITS = ["frame.cpp"]

LIB_DMANN = os.path.join(PKG, "libdmann.so")
LIB_ANNMAP = os.path.join(PKG, "libannmap.so")


def _cuda_home():
    import shutil
    nv = shutil.which(NVCC) or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nv)))


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(REPO, "include", "*.h")) + glob.glob(os.path.join(HOST, "*.hpp")))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src, fmad in CUDA_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([NVCC] + ARCH + COMMON + ["-fmad=" + ("true" if fmad else "false"),
                                                  "-Xptxas", "-v", "-c", s, "-o", o])
    for src in CXX_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([CXX, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I" + os.path.join(REPO, "include"), "-c", s, "-o", o])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if verbose:
        print("\n".join(logs))
    if force or _stale(LIB_DMANN, objs):
        _run([NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB_DMANN] + objs)
    host_srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if host_srcs and (force or _stale(LIB_ANNMAP, host_srcs + hdrs + [LIB_DMANN])):
        cuda = _cuda_home()
        _run([CXX, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
              "-I" + os.path.join(REPO, "include"), "-I" + HOST, "-I" + os.path.join(cuda, "include")] +
             host_srcs + ["-L" + PKG, "-ldmann", "-L" + os.path.join(cuda, "lib64"), "-lcudart",
                          "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(cuda, "lib64"),
                          "-o", LIB_ANNMAP])
    return LIB_DMANN


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB_DMANN)
