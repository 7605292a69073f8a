"""Builds libprgpu.so (sm_103a) and the prgpu command-line tool in-tree.

nvcc compiles each translation unit in parallel; the library is linked with the
static CUDA runtime.  Device code uses --fmad=false (every fused multiply-add is
explicit in the source) and host code -ffp-contract=off.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libprgpu.so")
CLI = os.path.join(HERE, "prgpu")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-Xptxas", "-O3"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off"]
SOURCES = ["api.cu", "octree.cu", "basis.cu", "rhs.cu", "solve.cu", "iso.cu", "noalloc.cu", "learned.cu", "flexcg.cu",
           "ply.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _needs(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "prgpu.h"))
    jobs, objs = [], []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _needs(obj, [path] + headers):
            if src.endswith(".cu"):
                jobs.append([NVCC] + CU_FLAGS + ["-c", path, "-o", obj])
            else:
                jobs.append(["g++"] + CXX_FLAGS + ["-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _needs(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs)
    cli_src = os.path.join(HERE, "cli", "prgpu_cli.cpp")
    if force or _needs(CLI, [cli_src, LIB]):
        _run(["g++", "-O2", "-std=c++17", cli_src, "-o", CLI, "-L" + HERE, "-lprgpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
