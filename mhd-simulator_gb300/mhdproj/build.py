"""Build recipe of libmhdproj.so: every CUDA translation unit is compiled for
sm_103a by nvcc in parallel, then linked into one shared library next to this
file.  No CMake, no torch extension: the library has a plain C ABI
(include/mhdproj.h)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(HERE, "libmhdproj.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
           "-I" + INCLUDE]
# Units whose FP32 arithmetic must follow the reference's operation order
# exactly: no fused multiply-adds.
EXACT = {"reference_kernels.cu", "step_kernels.cu", "em_solver.cu"}

SOURCES = ["context.cu", "gb300_kernels.cu", "fine_kernels.cu", "fused_kernels.cu", "tma_fused.cu", "mg_kernels.cu", "reference_kernels.cu", "noalloc.cu",
           "topology_kernels.cu", "step_kernels.cu", "export_fields.cu", "em_solver.cu",
           "classify.cu"]
HOST_SOURCES = ["topology.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmhdproj")


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))], HOST_SOURCES


def _deps():
    out = [os.path.join(INCLUDE, "mhdproj.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = _sources()
    jobs = []
    objs = []
    for s in cu:
        o = os.path.join(OBJ, s + ".o")
        flags = list(NVFLAGS) + (["-fmad=false"] if s in EXACT else [])
        jobs.append([nvcc, *ARCH, *flags, "-c", os.path.join(CSRC, s), "-o", o])
        objs.append(o)
    for s in cpp:
        o = os.path.join(OBJ, s + ".o")
        jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-I" + INCLUDE, "-c", os.path.join(CSRC, s), "-o", o])
        objs.append(o)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        for msg in ex.map(_compile, jobs):
            if verbose and msg:
                sys.stderr.write(msg)
    tmp = LIB + ".tmp"
    _compile([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
