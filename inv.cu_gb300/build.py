"""Builds libgbfwi.so (CUDA kernels + C ABI) and the gbinv command in-tree.

Every translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked with the
shared CUDA runtime and cuFFT. Outputs land next to this file:
    libgbfwi.so   the drop-in library (include/gbfwi.h)
    gbinv         the command-line driver (same arguments as inv.cu's main)
Usage: python inv.cu_gb300/build.py [--verbose] [--ptxas]
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
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbfwi.so")
EXE = os.path.join(HERE, "gbinv")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["gb_step.cu", "gb_march.cu", "gb_cluster.cu", "gb_aux.cu", "gb_misfit.cu", "gb_solver.cu", "gb_snapshot.cu", "gb_server.cu", "gb_abi.cu", "gb_config.cpp",
               "gb_optimizer.cpp"]
EXE_SOURCES = ["gbinv.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(ptxas: bool):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-Wall,-Wno-unused-function,-ffp-contract=off",
                "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src: str, ptxas: bool, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".h")]
    deps.append(os.path.join(ROOT, "include", "gbfwi.h"))
    if os.path.exists(obj) and not ptxas and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [_nvcc()] + _flags(ptxas) + ["-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if ptxas or verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, ptxas: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = LIB_SOURCES + EXE_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = dict(zip(srcs, ex.map(lambda s: _compile(s, ptxas, verbose), srcs)))
    lib_objs = [objs[s] for s in LIB_SOURCES]
    need_link = not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in lib_objs)
    if need_link:
        cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + lib_objs + ["-lcufft"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    if need_link or not os.path.exists(EXE):
        cmd = [_nvcc()] + ARCH + ["-cudart", "shared", "-o", EXE, objs["gbinv.cpp"], "-L", HERE, "-lgbfwi",
                                  "-Xlinker", "-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(verbose="--verbose" in sys.argv, ptxas="--ptxas" in sys.argv)
    print(LIB)
