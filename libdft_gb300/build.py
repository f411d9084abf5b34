"""Build libdftgpu.so in-tree for sm_103a (GB300).

Each CUDA translation unit is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a``; the C compatibility layer
(REAL complex entry points) is compiled by the host C compiler; everything is
linked into ``libdft_gb300/libdftgpu.so``.  Run ``python -m libdft_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdftgpu.so")
INCLUDE = os.path.join(ROOT, "include")

CU_SOURCES = ["fft.cu", "grid.cu", "ot.cu", "api.cu", "adjoint.cu", "noalloc.cu", "drivers.cu"]
C_SOURCES = ["compat.c", "maps.c"]

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    # host arithmetic without FMA contraction: the same results on x86 and Arm
    common = [ARCH, "-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I", INCLUDE, "-I", CSRC]
    if os.environ.get("DFTGPU_PTXAS_VERBOSE"):
        common += ["-Xptxas", "-v"]
    cmds = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        cmds.append([nv, *common, "-c", src, "-o", obj])
        objs.append(obj)
    cc = os.environ.get("CC", "gcc")
    for s in C_SOURCES:
        obj = os.path.join(BUILD, s.replace(".c", ".o"))
        cmds.append([cc, "-O2", "-fPIC", "-ffp-contract=off", "-std=gnu11", "-I", INCLUDE, "-c", os.path.join(CSRC, s), "-o", obj])
        objs.append(obj)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _run([nv, ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
