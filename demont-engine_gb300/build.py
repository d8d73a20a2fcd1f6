"""Builds the in-tree shared library libdemont_pt.so (CUDA kernels for
sm_103a + the C++ host scene builder) next to this file, under _build/.

    python demont-engine_gb300/build.py

nvcc compiles the .cu with -fmad=false (no FMA contraction: every float
expression rounds as written) and g++ compiles the host C++ with
-ffp-contract=off for the same reason.  The host scene builder is C++23; the
CUDA translation unit is C++20, the newest dialect nvcc 13 accepts.  One
-gencode, two translation units, compiled in parallel.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdemont_pt.so")
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", SRC]
    cu_obj = os.path.join(OUT, "pt_gpu.o")
    cpp_obj = os.path.join(OUT, "scene.o")
    jobs = [
        [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++20", "-fmad=false", "-prec-div=true",
         "-prec-sqrt=true", "-Xcompiler", "-fPIC,-ffp-contract=off", *inc, "-c",
         os.path.join(SRC, "pt_gpu.cu"), "-o", cu_obj],
        [CXX, "-std=c++23", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", *inc, "-c",
         os.path.join(SRC, "scene.cpp"), "-o", cpp_obj],
    ]
    with ThreadPoolExecutor(2) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    _run([NVCC, *ARCH, "-shared", "-o", LIB, cu_obj, cpp_obj, "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
