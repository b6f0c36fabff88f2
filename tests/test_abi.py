"""The C ABI libraries build, load and export every declared symbol; host-side
helpers behave as the reference's.  CPU only (no transform is run here)."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import HAS_GPU, REPO, PKG
from tests.golden.cases import make_input

HEADERS = [os.path.join(REPO, "include", h) for h in ("leg2cheb.h", "l2c_cuda.h")]


def _declared(path):
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"#define(?:[^\n]*\\\n)*[^\n]*", "", src)
    names = set()
    for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", src):
        name = m.group(1)
        if name in ("if", "while", "for", "return", "sizeof", "defined", "__has_include"):
            continue
        names.add(name)
    return names


def _exports(path):
    import subprocess

    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_every_declared_symbol_is_exported(lib):
    exported = _exports(os.path.join(PKG, "lib", "libleg2cheb.so")) | _exports(
        os.path.join(PKG, "lib", "libl2c_cuda.so"))
    declared = set()
    for h in HEADERS:
        declared |= _declared(h)
    assert "create_fmm" in declared and "l2c_gpu_execute" in declared
    missing = sorted(declared - exported)
    assert not missing, f"declared but not exported: {missing}"


def test_libraries_load(lib):
    lib.load()
    assert lib.cuda_abi().l2c_gpu_version().decode().startswith("l2c-gb300")


def test_lambda_host_bitwise(lib, golden):
    L = lib.load()
    z = golden["Lambda_z"]
    assert np.array_equal([L.Lambda(float(v)) for v in z], golden["Lambda"])
    assert np.array_equal([L.LambdaI(i) for i in range(256)], golden["LambdaI"])
    e = np.array([L._LambdaE(float(v)) for v in z])
    assert np.max(np.abs(e - golden["LambdaE"]) / golden["LambdaE"]) < 2e-15
    assert abs(L.Lambda(14.5) - L._LambdaE(14.5)) < 1e-15  # src/bin/l2c.c:698
    assert abs(L._Lambda0(24.5) - 0.20100243720317808186742632) < 1e-14
    w = np.zeros(5)
    zz = np.array([0.0, 0.5, 3.25, 12.0, 99.5])
    L.Lambdavec(zz.ctypes.data, w.ctypes.data, 5)
    assert np.array_equal(w, [L.Lambda(v) for v in zz])


def _matvectri_ref(A, x, m, upper, b0=None):
    """numpy statement of leg2cheb.c:537-619 semantics."""
    if not upper:
        b = np.zeros(m)
        k = 0
        for i in range(m):
            for j in range(i + 1):
                z = x[j] + x[m + j] if (i + j) % 2 == 0 else x[j] - x[m + j]
                b[i] += A[k] * z
                k += 1
        return b
    b = b0.copy()
    k = 0
    for i in range(m):
        se = so = 0.0
        for j in range(i, m):
            if (j - i) % 2 == 0:
                se += A[k] * x[j]
            else:
                so += A[k] * x[j]
            k += 1
        b[i] += se + so
        b[m + i] += se - so
    return b


@pytest.mark.parametrize("m", [18, 17, 6])
@pytest.mark.parametrize("upper", [False, True])
def test_matvectri(lib, m, upper):
    L = lib.load()
    rng = np.random.default_rng(m)
    A = rng.standard_normal((m * m + m) // 2)
    x = rng.standard_normal(2 * m)
    b0 = rng.standard_normal(2 * m)
    b = b0.copy()
    L.matvectri(A.ctypes.data, x.ctypes.data, b.ctypes.data, m, upper)
    want = _matvectri_ref(A, x, m, upper, b0)
    if not upper:
        assert np.allclose(b[:m], want, rtol=1e-14, atol=1e-14)
    else:
        assert np.allclose(b, want, rtol=1e-14, atol=1e-14)


def test_matvectri_reproduces_binomial_transfer(lib, golden):
    # with the exact tables, the lower product maps two children to the parent
    L = lib.load()
    B = np.array(golden["BMe"])
    x = make_input(36, "gauss", 3)
    b = np.zeros(36)
    L.matvectri(B.ctypes.data, x.ctypes.data, b.ctypes.data, 18, False)
    assert np.allclose(b[:18], _matvectri_ref(B, x, 18, False), rtol=1e-14, atol=1e-15)


def test_dct2(lib):
    L = lib.load()
    X = np.random.default_rng(3).standard_normal(324)
    out = np.zeros(324)
    L.dct2(X.ctypes.data, out.ctypes.data)
    k = np.arange(18)[:, None]
    n = np.arange(18)[None, :]
    C = np.cos(np.pi * k * (n + 0.5) / 18)
    E = C @ X.reshape(18, 18) @ C.T / 81
    E[0, :] *= 0.5
    E[:, 0] *= 0.5
    assert np.max(np.abs(out.reshape(18, 18) - E)) < 1e-14


def test_tree_helpers(lib):
    L = lib.load()
    for f in ("get_number_of_blocks", "get_total_number_of_blocks", "get_number_of_submatrices",
              "get_total_number_of_submatrices"):
        getattr(L, f).restype = ctypes.c_size_t
        getattr(L, f).argtypes = [ctypes.c_size_t]
    L.get_h.restype = ctypes.c_size_t
    L.get_h.argtypes = [ctypes.c_size_t, ctypes.c_size_t]
    for lv in range(12):
        assert L.get_number_of_blocks(lv) == 2 ** (lv + 1) - 1
        assert L.get_total_number_of_blocks(lv + 1) == 2 ** (lv + 2) - (lv + 3)
        assert L.get_number_of_submatrices(lv) == 3 * (2 ** (lv + 1) - 1)
    assert L.get_h(0, 5) == 16 and L.get_h(4, 5) == 1
    ij = (ctypes.c_size_t * 2)()
    L.get_ij.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t,
                         ctypes.c_size_t]
    L.get_ij(ij, 2, 3, 64, 6)
    assert (ij[0], ij[1]) == (2 * 3 * 64 * 8, 2 * 3 * 64 * 8 + 2 * 64 * 8)


def test_geometry_degenerate(lib):
    # no levels, and no arithmetic on log(0) or a division by zero
    assert lib.geometry(0, 64) == (0, 0, 0)
    assert lib.geometry(1000, 0) == (0, 0, 1000)
    assert lib.geometry(1, 64) == (0, 0, 1)


@pytest.mark.parametrize("N", [20, 256, 257, 300, 512, 1000, 1024, 4097, 65536, 1 << 20, 1 << 24])
@pytest.mark.parametrize("maxs", [32, 36, 50, 64])
def test_geometry_matches_oracle(lib, orc, N, maxs):
    L, s, Nn = lib.geometry(N, maxs)
    o = orc.Oracle(min(N, 1 << 12), maxs, 0) if N <= 4096 else None
    # closed form of leg2cheb.c:860-871
    import math

    Lr = math.ceil(math.log2(N / maxs)) - 2
    if Lr < 1:
        assert L == 0
    else:
        assert L == Lr
        assert s == math.ceil(N / 2 ** (Lr + 2))
        assert Nn == s * 2 ** (Lr + 2)
    if o is not None:
        assert (o.L, o.s if o.L else 0) == (L, s if L else 0)


@pytest.mark.skipif(HAS_GPU, reason="checks the no-GPU failure path")
def test_fails_loudly_without_gpu(lib):
    L = lib.load()
    p = L.create_fmm(1024, 64, 18, 2, 0, 0, 0)
    assert not p
    assert "cuda" in lib.last_error().lower() or "device" in lib.last_error().lower()
    with pytest.raises(lib.L2CError):
        lib.Plan(1024, 64)


def test_rejects_unsupported_forms(lib):
    with pytest.raises(lib.L2CError, match="M = 18"):
        lib.Plan(1024, 64, M=20)
    with pytest.raises(lib.L2CError, match="lagrange must be 0"):
        lib.Plan(1024, 64, lagrange=2)
    # ragged lists: modal form only, refused before any device work
    import ctypes

    import numpy as np

    L = lib.load()
    Ns = np.array([1000, 5000], dtype=np.uint64)
    assert not L.create_fmm_ragged(2, ctypes.c_void_p(Ns.ctypes.data), 64, 18, 2, 1, 0, 0)
    assert "modal form" in lib.last_error()
