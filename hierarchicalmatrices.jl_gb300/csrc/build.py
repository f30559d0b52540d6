"""Builds libhmgpu.so (sm_103a CUDA + C++ host planner) in-tree.

    python hierarchicalmatrices.jl_gb300/csrc/build.py [--force]

Objects go to hierarchicalmatrices.jl_gb300/_build/, the library to
hierarchicalmatrices.jl_gb300/lib/libhmgpu.so.  Translation units compile in
parallel; the CUDA runtime is linked statically.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

CSRC = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(CSRC)
REPO = os.path.dirname(PKG_ROOT)
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB = os.path.join(LIB_DIR, "libhmgpu.so")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["hm_kernels.cu", "hm_ring.cu", "hm_df.cu", "hm_wide.cu", "hm_blocks.cu", "hm_tc.cu", "hm_algebra.cu", "hm_api.cu"]
CPP_SOURCES = ["hm_plan.cpp"]
HEADERS = ["hm_types.h", "hm_plan.h", "hm_kernels.cuh", "hm_async.cuh"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def build(force=False, verbose=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "hmgpu.h")]
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-static-global-template-stub=false",
                         "-I", CSRC, "-I", INCLUDE, "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-Wall", "-I", CSRC, "-I", INCLUDE,
                         "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
