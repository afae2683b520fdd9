"""Builds libtroute_gb300.so in-tree (sm_103a, no CMake, parallel compile).

The CUDA translation unit is compiled by nvcc for sm_103a only; the host
translation units by g++ with -ffp-contract=off so the derived per-segment
values and the seeded generator round identically on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
# TROUTE_BUILD_DIR / TROUTE_LIB_DIR place a variant build (e.g. the
# self-checking one, TROUTE_CHECK=1) beside the default one
BUILD = os.environ.get("TROUTE_BUILD_DIR") or os.path.join(PKG_ROOT, "_build")
LIBDIR = os.environ.get("TROUTE_LIB_DIR") or os.path.join(PKG_ROOT, "lib")
LIB = os.path.join(LIBDIR, "libtroute_gb300.so")
INCLUDE = os.path.join(os.path.dirname(PKG_ROOT), "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["kernels.cu", "route_pool.cu", "route_dataflow.cu", "noalloc.cu", "warm.cu", "warm_gemm.cu", "linear.cu",
              "diffusive.cu", "matrix.cu"]
CPP_SOURCES = ["network.cpp", "capi.cpp", "gen.cpp", "netfile.cpp", "forcing.cpp"]


def _sources():
    return [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES]


def _deps():
    out = _sources()
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    out.append(os.path.join(INCLUDE, "troute_gb300.h"))
    out.append(os.path.abspath(__file__))
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles and links the library; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cuda_inc = os.path.join(CUDA_HOME, "include")
    jobs = []
    objs = []
    # No implicit FMA contraction: the solver then rounds every +, -, *, / like
    # the reference's C on the host (explicit fma() calls are unaffected).
    fmad = ["-fmad=false"] if os.environ.get("TROUTE_FMAD", "0") == "0" else []
    # TROUTE_CHECK=1: self-checking kernels (dependency and bounds invariants are
    # verified on the device and reported as errors instead of being assumed)
    if os.environ.get("TROUTE_CHECK", "0") == "1":
        fmad = fmad + ["-DTROUTE_CHECK"]
    fmad = fmad + [f"-D{d}" for d in os.environ.get("TROUTE_DEFINES", "").split() if d]
    for f in CU_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append([NVCC, *ARCH, *fmad, "-O3", "-lineinfo", "-std=c++17", "-Xptxas", "-v",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE,
                     "-c", os.path.join(CSRC, f), "-o", o])
    for f in CPP_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                     "-I", INCLUDE, "-I", cuda_inc, "-c", os.path.join(CSRC, f), "-o", o])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            sys.stdout.write(lg)
    tmp = LIB + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, LIB)
    # keep the ptxas report next to the objects (registers / spills per kernel)
    with open(os.path.join(BUILD, "ptxas.txt"), "w") as fh:
        fh.write("".join(logs[: len(CU_SOURCES)]))
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
