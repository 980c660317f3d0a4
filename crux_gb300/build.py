"""Build the GB300 library in-tree: crux_gb300/_lib/libcxlik_gpu.so.

nvcc compiles each translation unit (host-only .cpp files too) for sm_103a only (arch-specific
``compute_103a``), in parallel, then links one shared library.  Usage:
``python -m crux_gb300.build`` (or ``__graft_entry__.build()``).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libcxlik_gpu.so")
SOURCES = ["cxg_kernels.cu", "cxg_lik.cu", "cxg_noalloc.cu", "cxg_mc3.cu",
           "cxg_serve.cu", "cxg_compact.cu", "cxg_plan.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-O3", "-I" + os.path.join(ROOT, "include"),
         "-I" + SRC]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(SRC, f) for f in os.listdir(SRC)
                    if f.endswith((".h", ".cuh"))] + [os.path.join(ROOT, "include",
                                                          "cxlik_gpu.h")]
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    objs = []

    def one(src):
        s = os.path.join(SRC, src)
        o = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        if _stale(o, s):
            cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd))
            subprocess.run(cmd, check=True)
        return o

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB)
                                      for o in objs):
        # -ldl: the header-only NVTX ranges open a profiler's injection
        # library on demand.
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart",
               "-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
