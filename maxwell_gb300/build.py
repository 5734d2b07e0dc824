"""Builds libmaxwell_gb300.so in-tree for sm_103a (nvcc + gcc, no cmake).

    python -m maxwell_gb300.build      # or __graft_entry__.build()
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmaxwell_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc") if os.path.exists(os.path.join(CUDA, "bin", "nvcc")) else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["mx_stencil.cu", "mx_dense.cu", "mx_block.cu", "mx_vec.cu", "mx_nodegs.cu"]
C = ["mx_abi.c", "mx_solver.c", "mx_kbench.c"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return cmd[-1]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "maxwell_gb300.h"))
    jobs, objs = [], []
    for f in CU:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([NVCC, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-I", SRC, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj])
    for f in C:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-Wall", "-I", SRC, "-I", os.path.join(ROOT, "include"),
                         "-I", os.path.join(CUDA, "include"), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for done in ex.map(_run, jobs):
            if verbose:
                print("built", done)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lm"])
        shutil.move(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
