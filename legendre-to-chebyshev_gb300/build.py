"""Build the in-tree shared libraries.

    lib/libl2c_cuda.so   sm_103a kernels + C ABI (include/l2c_cuda.h)   [nvcc]
    lib/libleg2cheb.so   the reference's public C API (include/leg2cheb.h),
                         linked against libl2c_cuda.so with an $ORIGIN rpath [gcc]

Run ``python build.py`` (or call build()).  Rebuilds only what is out of date.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CUDA_SOURCES = [os.path.join(CSRC, "l2c_cuda.cu")]
CUDA_DEPS = CUDA_SOURCES + [os.path.join(CSRC, f) for f in ("l2c_lambda.h", "l2c_tables.h", "l2c_ozaki.cuh", "l2c_tc.cuh")] + [
    os.path.join(INCLUDE, "l2c_cuda.h")
]
HOST_SOURCES = [os.path.join(CSRC, "leg2cheb_host.c")]
HOST_DEPS = HOST_SOURCES + [os.path.join(INCLUDE, f) for f in ("leg2cheb.h", "l2c_cuda.h")] + [
    os.path.join(CSRC, "l2c_tables.h")
]

CUDA_LIB = os.path.join(LIB, "libl2c_cuda.so")
HOST_LIB = os.path.join(LIB, "libleg2cheb.so")


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force=False, verbose=False):
    os.makedirs(LIB, exist_ok=True)
    if force or _stale(CUDA_LIB, CUDA_DEPS):
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-shared",
               "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE,
               "-o", CUDA_LIB + ".tmp", *CUDA_SOURCES]
        out = _run(cmd)
        os.replace(CUDA_LIB + ".tmp", CUDA_LIB)
        if verbose:
            print(out)
    if force or _stale(HOST_LIB, HOST_DEPS + [CUDA_LIB]):
        cc = os.environ.get("CC", "gcc")
        cmd = [cc, "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
               "-Wl,-soname,libleg2cheb.so",
               "-I", INCLUDE, "-o", HOST_LIB + ".tmp", *HOST_SOURCES,
               "-L", LIB, "-l:libl2c_cuda.so", "-Wl,-rpath,$ORIGIN", "-lm"]
        out = _run(cmd)
        os.replace(HOST_LIB + ".tmp", HOST_LIB)
        if verbose:
            print(out)
    return HOST_LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print("built", CUDA_LIB, HOST_LIB)
