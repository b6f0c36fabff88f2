"""Golden-vector cases: name -> (N, maxs, direction, stride, distribution, seed).

Distributions follow the workloads the transform is benchmarked on:
  uniform  : iid U[-1, 1]                       (single vector N = 512, ragged lists)
  sign     : s_n / (n + 1), s_n iid +-1          (single vectors N = 2^k)
  gauss2   : iid N(0, 1) * (n + 1)^-2            (lines of a 64x64x1024 array)
  gauss    : iid N(0, 1)                         (mixed-precision cases)
  ones     : all ones                            (src/bin/l2c.c:84-86 known answers)
"""
import numpy as np


def make_input(n, dist, seed):
    rng = np.random.default_rng(seed)
    idx = np.arange(n, dtype=np.float64)
    if dist == "uniform":
        return rng.uniform(-1.0, 1.0, n)
    if dist == "sign":
        return rng.choice([-1.0, 1.0], n) / (idx + 1.0)
    if dist == "gauss2":
        return rng.standard_normal(n) / (idx + 1.0) ** 2
    if dist == "gauss":
        return rng.standard_normal(n)
    if dist == "ones":
        return np.ones(n)
    raise ValueError(dist)


def _cases():
    c = {}
    # direct path (L < 1): N <= 4 maxs
    for N, maxs in ((20, 64), (100, 32), (255, 64), (256, 64)):
        for d in (0, 1):
            for st in (1, 3):
                c[f"direct_N{N}_s{maxs}_d{d}_st{st}"] = (N, maxs, d, st, "uniform", 11 + N)
    c["ones_N20_s64_d0_st1"] = (20, 64, 0, 1, "ones", 0)
    c["ones_N20_s64_d1_st1"] = (20, 64, 1, 1, "ones", 0)
    # FMM path: level counts 1..8, both leaf sizes the reference uses
    fmm = [(258, 64), (300, 64), (512, 64), (512, 32), (1000, 36), (1024, 64), (2000, 64),
           (4096, 64), (4096, 32), (6000, 50), (16384, 64), (16384, 32), (65536, 64)]
    for N, maxs in fmm:
        for d in (0, 1):
            for dist in (("uniform", "sign") if N < 16384 else ("sign",)):
                c[f"fmm_N{N}_s{maxs}_d{d}_st1_{dist}"] = (N, maxs, d, 1, dist, 100 + N + d)
    for N, maxs in ((512, 64), (1024, 64), (4096, 32)):
        for d in (0, 1):
            c[f"fmm_N{N}_s{maxs}_d{d}_st3_gauss2"] = (N, maxs, d, 3, "gauss2", 200 + N + d)
    c["fmm_N1024_s64_d0_st1_gauss2"] = (1024, 64, 0, 1, "gauss2", 5)
    c["fmm_N1024_s64_d1_st1_gauss2"] = (1024, 64, 1, 1, "gauss2", 5)
    c["fmm_N16384_s64_d0_st1_gauss"] = (16384, 64, 0, 1, "gauss", 6)
    c["fmm_N16384_s64_d1_st1_gauss"] = (16384, 64, 1, 1, "gauss", 6)
    # odd N: C2L only (reference L2C runs past its arrays for odd N, L >= 1)
    for N, maxs in ((257, 64), (1023, 64), (5001, 64)):
        c[f"fmm_N{N}_s{maxs}_d1_st1_uniform"] = (N, maxs, 1, 1, "uniform", 300 + N)
    return c


CASES = _cases()


def _nodal_cases():
    """Nodal form (create_fmm with lagrange = 1): FMM path only (the direct
    path does not depend on the form)."""
    c = {}
    for N, maxs in ((512, 64), (1024, 64), (4096, 32), (6000, 50), (16384, 64)):
        for d in (0, 1):
            for dist in ("uniform", "sign"):
                c[f"nodal_N{N}_s{maxs}_d{d}_st1_{dist}"] = (N, maxs, d, 1, dist, 400 + N + d)
    for d in (0, 1):
        c[f"nodal_N1024_s64_d{d}_st3_gauss2"] = (1024, 64, d, 3, "gauss2", 500 + d)
    c["nodal_N1023_s64_d1_st1_uniform"] = (1023, 64, 1, 1, "uniform", 601)
    return c


NODAL_CASES = _nodal_cases()
