"""Builds libnbounce.so in-tree for sm_103a.

Host C++ (BVH builder, Sobol generator) is compiled with the host compiler and
-ffp-contract=off (the builder reproduces Rust's uncontracted f32 arithmetic); the CUDA
translation units with nvcc for ``-gencode arch=compute_103a,code=sm_103a`` and
-fmad=false / IEEE division and square root (the kernels follow the same arithmetic
contract as the CPU oracle).  Objects are compiled in parallel; the shared library links
the CUDA runtime statically.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnbounce.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "--expt-relaxed-constexpr",
              "-I", CSRC, "-I", INCLUDE]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-Wall",
             "-I", CSRC, "-I", INCLUDE]
CU_SOURCES = ["nb_kernels.cu", "nb_api.cu", "nb_server.cu", "nb_static.cu", "nb_cache.cu", "nb_bc6h.cu"]
CXX_SOURCES = ["nb_scene.cpp", "nb_sobol.cpp"]
HEADERS = ["nb_internal.h", "nb_device.cuh", "nb_launch.h", "nb_runtime.h", "nb_mlp.cuh", "sobol_directions.inc"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_nvcc=()):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "nbounce.h"), __file__]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, *extra_nvcc, "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([os.environ.get("CXX", "g++"), *CXX_FLAGS, "-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        run([nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
