"""The nodal (Lagrange) form, create_fmm(..., lagrange = 1, ...): leaf matrices
of barycentric interpolation weights (leg2cheb.c:997-1031), far-field blocks of
kernel samples (no DCT, leg2cheb.c:938, 973), transfer matrices B0 | B1
(leg2cheb.c:1076-1100) in both tree sweeps (leg2cheb.c:1401-1416, 1450-1464).
Same 1e-14 relative max-norm bar as the modal form, against golden vectors
from the reference run with lagrange = 1, the oracle's nodal port and the
extended-precision direct sum."""
import numpy as np
import pytest

from oracle import direct_ld
from tests.conftest import relerr
from tests.golden.cases import NODAL_CASES, make_input

pytestmark = pytest.mark.gpu

TOL = 1e-14


@pytest.mark.parametrize("key", sorted(NODAL_CASES))
def test_nodal_golden_cases(lib, golden, key):
    N, maxs, d, st, dist, seed = NODAL_CASES[key]
    u = make_input(N * st, dist, seed)
    out = np.zeros(N * st)
    p = lib.Plan(N, maxs, direction=2, lagrange=1)
    flops = p.execute(u, out, d, st)
    assert flops == int(golden[key + "/flops"])
    assert relerr(out, golden[key + "/out"]) <= TOL


def test_nodal_plan_tables(lib, orc, golden):
    p = lib.Plan(1024, 64, lagrange=1)
    # host-side libm arithmetic, as the reference: bit for bit
    assert np.array_equal(p.copy_table(5), golden["nodal_plan_N1024_s64/T"])
    assert np.array_equal(p.copy_table(6), golden["nodal_plan_N1024_s64/B"])
    o = orc.Oracle(1024, 64, 2, lagrange=1)
    for d in (0, 1):
        A = p.copy_table(d).reshape(-1, 18, 18)
        B = o.A(d).reshape(-1, 18, 18)
        err = np.max(np.abs(A - B), axis=(1, 2)) / np.max(np.abs(B), axis=(1, 2))
        assert err.max() < 1e-14
    assert len(lib.Plan(1024, 64).copy_table(6)) == 0  # modal plans have none


@pytest.mark.parametrize("N,maxs", [(1 << 16, 32), (1 << 20, 64), (100001, 64)])
@pytest.mark.parametrize("d", [0, 1])
def test_nodal_large_vs_oracle(lib, orc, N, maxs, d):
    if N % 2 and d == 0:
        pytest.skip("odd-N L2C is covered by the modal tests; the form does not change it")
    u = make_input(N, "sign", N + d)
    p = lib.Plan(N, maxs, lagrange=1)
    out = np.zeros(N)
    flops = p.execute(u, out, d)
    o = orc.Oracle(N, maxs, 2, lagrange=1)
    want = np.zeros(N)
    assert flops == o.execute(u, want, d)
    assert relerr(out, want) <= TOL


def test_nodal_vs_extended_precision(lib):
    N = 8192
    u = make_input(N, "uniform", 3)
    p = lib.Plan(N, 32, lagrange=1)
    for d, f in ((0, direct_ld.l2c_direct), (1, direct_ld.c2l_direct)):
        out = np.zeros(N)
        p.execute(u, out, d)
        assert direct_ld.rel_maxnorm(out, f(u)) < 5e-15


@pytest.mark.parametrize("count,N,maxs", [(64, 1024, 64), (16, 16384, 32)])
def test_nodal_batched_and_round_trip(lib, orc, count, N, maxs):
    x = np.ascontiguousarray(make_input(N * count, "gauss2", 8).reshape(count, N))
    p = lib.Plan(N, maxs, lagrange=1)
    o = orc.Oracle(N, maxs, 2, lagrange=1)
    c = np.zeros_like(x)
    p.execute_batched(x, c, 0, count, N, 1)
    for i in (0, count - 1):
        assert relerr(c[i], o(x[i], 0)[:N]) <= TOL
    b = np.zeros_like(x)
    p.execute_batched(c, b, 1, count, N, 1)
    assert relerr(b, x) <= 1e-13


def test_nodal_precompute_and_2d(lib, orc):
    N0, N1 = 64, 2048
    x = np.ascontiguousarray(make_input(N0 * N1, "gauss", 4).reshape(N0, N1))
    out = np.zeros_like(x)
    lib.Plan2D(N0, N1, 1, maxs=32, lagrange=1, precompute=1)(x, out, 0)
    o = orc.Oracle(N1, 32, 2, lagrange=1)
    for r in (0, N0 - 1):
        assert relerr(out[r], o(x[r], 0)[:N1]) <= TOL


def test_nodal_rejects_mixed(lib):
    with pytest.raises(lib.L2CError, match="modal form only"):
        lib.Plan(16384, 16, lagrange=1, mixed=True)
