"""Builds libmorgana_gpu.so in-tree for sm_103a.

The CUDA sources are compiled with nvcc (-gencode arch=compute_103a,code=sm_103a)
and the host C++ with g++, in parallel, then linked into
morganapublic_gb300/_build/libmorgana_gpu.so.  Rebuilds only what changed.
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
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmorgana_gpu.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["mg_assemble.cu", "mg_solve.cu", "mg_pattern.cu", "mg_lagrange.cu", "mg_schedule.cu"]
CPP_SOURCES = ["mg_mesh.cpp", "mg_plan.cpp", "mg_lagrange.cpp"]


def _newer(src_paths, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in src_paths)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles and links the library; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in sorted(os.listdir(CSRC)) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "morgana_gpu.h"))
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            jobs.append([NVCC, "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-fopenmp", "-I" + INCLUDE, "-I" + CSRC,
                         "-c", src, "-o", obj])
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-Wall",
                         "-I" + os.path.join(CUDA_HOME, "include"), "-I" + INCLUDE, "-I" + CSRC,
                         "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or _newer(objs, LIB):
        tmp = LIB + ".tmp"
        _run([NVCC, "-shared", *ARCH, "-o", tmp, *objs, "-Xcompiler", "-fopenmp",
              "--cudart", "shared", "-Xlinker", "-rpath=" + os.path.join(CUDA_HOME, "lib64")])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
