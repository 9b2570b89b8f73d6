"""In-tree build of libephgb.so (the CUDA kernels, the host side and the C
ABI of include/eph_gb.h) for sm_103a.  Plain nvcc/g++ calls, run in
parallel; the library lands next to this package (user-eph_gb300/)."""
from __future__ import annotations

import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)  # user-eph_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(ROOT, "libephgb.so")

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# no floating-point contraction anywhere: EXACT mode must round like the
# reference's source expressions; FAST mode writes its fma() calls explicitly
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I" + INCLUDE] + os.environ.get("EPH_NVCC_FLAGS", "").split()
CXX_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-std=c++17", "-I" + INCLUDE]

SOURCES = [("eph_ctx.cu", "nvcc"), ("eph_adjoint.cu", "nvcc"), ("eph_eam.cu", "nvcc"), ("eph_noalloc.cu", "nvcc"), ("eph_host.cpp", "cxx")]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(INCLUDE, "eph_gb.h"))
    procs, objs = [], []
    for src, tool in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not force and not _newer(o, [s] + headers):
            continue
        cmd = ([NVCC] + NVCC_FLAGS if tool == "nvcc" else [CXX] + CXX_FLAGS) + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + out.decode(errors="replace"))
    if force or _newer(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
