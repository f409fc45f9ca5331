"""Builds libwvgpu.so (CUDA kernels + C ABI) for sm_103a, in-tree.

Host C++ is compiled with g++ (-ffp-contract=off: the descriptor's mode order
depends on unfused k*k + l*l), CUDA with nvcc -gencode arch=compute_103a,
code=sm_103a.  Translation units compile in parallel; the library is rebuilt
only when a source is newer than it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "build")
LIB = os.path.join(HERE, "libwvgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SOURCES = ["wv_descriptor.cpp", "wv_plan.cpp"]
CUDA_SOURCES = ["wv_api.cu", "wv_rk23.cu", "wv_system.cu"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    out = []
    for name in os.listdir(CSRC):
        if name.endswith((".cpp", ".cu", ".cuh", ".hpp", ".h")):
            out.append(os.path.join(CSRC, name))
    out.append(os.path.join(INCLUDE, "wvgpu.h"))
    out.append(os.path.abspath(__file__))
    return out


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(force=False, verbose=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}", "-c",
                     os.path.join(CSRC, src), "-o", obj])
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        jobs.append([nvcc, "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}", "-c", os.path.join(CSRC, src), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, len(jobs))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
    tmp = LIB + ".tmp"
    _run([nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lrt", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
