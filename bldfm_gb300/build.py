"""Build libbldfm_gb300.so in-tree for sm_103a (nvcc + gcc, no cmake).

Usage: python -m bldfm_gb300.build  (or bldfm_gb300.build.build()).
Compiles each translation unit in parallel, then links one shared library.
"""

import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(HERE, "libbldfm_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

CU_SOURCES = ["api.cu", "geometry.cu", "xform.cu", "kernels.cu", "profiles.cu", "noalloc.cu", "batch.cu", "surrogate.cu", "serve.cu", "measure.cu"]
C_SOURCES = ["host_exact.c"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _needs(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "bldfm_gb300.h"))
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + headers):
            jobs.append(
                [NVCC, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                 "--expt-relaxed-constexpr", "-Xptxas", "-v" if verbose else "-O3",
                 "-c", src, "-o", obj]
            )
    for s in C_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + headers):
            # -fno-builtin: every libm call (pow, csqrt) runs in the library at
            # run time, as numpy's scalar ** and complex sqrt do; gcc would
            # otherwise fold pow(x, 2.0) into x * x, which differs from libm's
            # pow by one ulp for rare x
            jobs.append(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-fno-builtin", "-std=gnu11", "-c", src, "-o",
                         obj])
    outs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
    stamp = os.path.join(BUILD, "lib.stamp")
    if force or jobs or not os.path.exists(LIB) or not os.path.exists(stamp) or _needs(LIB, objs):
        _run([NVCC, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt", "-lm"])
        open(stamp, "w").write(platform.machine())
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
