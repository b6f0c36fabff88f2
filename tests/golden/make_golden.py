"""Generate golden vectors by running the UNMODIFIED reference.

Needs the reference built into oracle/_ref by ``make -C oracle ref`` (from the
reference tree given as REF=..., by default ``reference`` beside this
repository's root directory).  Writes tests/golden/golden.npz, committed so the
tests run without the reference (on the GPU machine it does not exist).

Contents (all produced by the reference's own code):
  * BMe / BMeT (leg2cheb.c:6-123), LambdaI(0..255), Lambda(z) at chosen z,
    _LambdaE(z) (lambda.c:51-63)
  * execute() outputs and flop counts for a list of (N, maxs, direction,
    stride, distribution, seed) cases, inputs regenerated from the seed.
  * the reference's round-trip (L2C then C2L, like `l2c -N512 -d2`)
  * nodal form (lagrange = 1): execute() outputs and flop counts for
    NODAL_CASES, and the plan's T and B (fmm_plan fields, leg2cheb.h:58-78)
    for N = 1024, maxs = 64

Output buffers handed to the reference carry 8 doubles of slack: for odd N
its parity scatter writes one element past the end (leg2cheb.c:1473-1476).
L2C with odd N and L >= 1 is not generated: the reference's last-block loop
(leg2cheb.c:283-294) runs past its arrays there.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from tests.golden.cases import CASES, NODAL_CASES, make_input  # noqa: E402

LIB = os.path.join(REPO, "oracle", "_ref", "libleg2cheb_ref.so")


def main():
    ref = ctypes.CDLL(LIB)
    ref.create_fmm.restype = ctypes.c_void_p
    ref.create_fmm.argtypes = [ctypes.c_size_t] * 7
    ref.free_fmm.argtypes = [ctypes.c_void_p]
    ref.execute.restype = ctypes.c_size_t
    ref.execute.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_size_t] * 2
    for name in ("Lambda", "_LambdaE"):
        getattr(ref, name).restype = ctypes.c_double
        getattr(ref, name).argtypes = [ctypes.c_double]
    ref.LambdaI.restype = ctypes.c_double
    ref.LambdaI.argtypes = [ctypes.c_size_t]

    out = {}
    out["BMe"] = np.array((ctypes.c_double * 171).in_dll(ref, "BMe"))
    out["BMeT"] = np.array((ctypes.c_double * 171).in_dll(ref, "BMeT"))
    out["LambdaI"] = np.array([ref.LambdaI(i) for i in range(256)])
    z = np.concatenate([np.arange(0, 12, 0.25), [14.5, 15.0, 20.5, 24.5, 40.5, 41.0, 100.3,
                                                 141.5, 142.0, 500.25, 2014.5, 3000.1, 1e6 + 0.5]])
    out["Lambda_z"] = z
    out["Lambda"] = np.array([ref.Lambda(float(v)) for v in z])
    out["LambdaE"] = np.array([ref._LambdaE(float(v)) for v in z])

    for key, (N, maxs, direction, stride, dist, seed) in CASES.items():
        u = make_input(N * stride, dist, seed)
        plan = ref.create_fmm(N, maxs, 18, 2, 0, 0, 0)
        o = np.zeros(N * stride + 8)
        flops = ref.execute(u.ctypes.data, o.ctypes.data, plan, direction, stride)
        ref.free_fmm(plan)
        out[key + "/out"] = o[: N * stride].copy()
        out[key + "/flops"] = np.array(flops, dtype=np.uint64)

    # Round trip like `l2c -N512 -d2` (src/bin/l2c.c:10-65) on U[-1,1] input
    for N, maxs in ((512, 64), (512, 32)):
        u = make_input(N, "uniform", 7)
        plan = ref.create_fmm(N, maxs, 18, 2, 0, 0, 0)
        c = np.zeros(N + 8)
        b = np.zeros(N + 8)
        ref.execute(u.ctypes.data, c.ctypes.data, plan, 0, 1)
        ref.execute(c.ctypes.data, b.ctypes.data, plan, 1, 1)
        ref.free_fmm(plan)
        out[f"roundtrip_{N}_{maxs}/cheb"] = c[:N].copy()
        out[f"roundtrip_{N}_{maxs}/leg"] = b[:N].copy()

    for key, (N, maxs, direction, stride, dist, seed) in NODAL_CASES.items():
        u = make_input(N * stride, dist, seed)
        plan = ref.create_fmm(N, maxs, 18, 2, 1, 0, 0)
        o = np.zeros(N * stride + 8)
        flops = ref.execute(u.ctypes.data, o.ctypes.data, plan, direction, stride)
        ref.free_fmm(plan)
        out[key + "/out"] = o[: N * stride].copy()
        out[key + "/flops"] = np.array(flops, dtype=np.uint64)

    # nodal plan data: fmm_plan is 7 size_t (direction, M, N, Nn, L, s,
    # lagrange), then double **A, double *T, double *B, double *BT
    plan = ref.create_fmm(1024, 64, 18, 2, 1, 0, 0)
    fields = (ctypes.c_void_p * 11).from_address(plan)
    s = ctypes.cast(plan + 5 * 8, ctypes.POINTER(ctypes.c_size_t))[0]
    Tp = ctypes.cast(fields[8], ctypes.POINTER(ctypes.c_double))
    Bp = ctypes.cast(fields[9], ctypes.POINTER(ctypes.c_double))
    out["nodal_plan_N1024_s64/T"] = np.ctypeslib.as_array(Tp, (2 * s * 18,)).copy()
    out["nodal_plan_N1024_s64/B"] = np.ctypeslib.as_array(Bp, (2 * 324,)).copy()
    ref.free_fmm(plan)

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
