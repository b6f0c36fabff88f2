"""The oracle port (oracle/l2c_oracle.c) pinned against the reference.

Golden vectors come from running the unmodified reference
(tests/golden/make_golden.py); known answers are the reference's own
(src/bin/l2c.c:69-74 and 695-707).  CPU only."""
import numpy as np
import pytest

from oracle import direct_ld
from tests.conftest import relerr
from tests.golden.cases import CASES, NODAL_CASES, make_input

# the port follows the reference's arithmetic; differences come only from the
# DCT and BLAS summation order (~1e-16)
PORT_TOL = 1e-14


@pytest.mark.parametrize("key", sorted(CASES))
def test_oracle_matches_reference_execute(orc, golden, key):
    N, maxs, d, st, dist, seed = CASES[key]
    u = make_input(N * st, dist, seed)
    o = orc.Oracle(N, maxs, 2)
    out = np.zeros(N * st)
    flops = o.execute(u, out, d, st)
    ref = golden[key + "/out"]
    assert flops == int(golden[key + "/flops"])
    assert relerr(out, ref) <= PORT_TOL


@pytest.mark.parametrize("key", sorted(NODAL_CASES))
def test_nodal_oracle_matches_reference_execute(orc, golden, key):
    # nodal form (lagrange = 1): the same transform through Lagrange
    # interpolation on the Chebyshev points instead of Chebyshev coefficients
    N, maxs, d, st, dist, seed = NODAL_CASES[key]
    u = make_input(N * st, dist, seed)
    o = orc.Oracle(N, maxs, 2, lagrange=1)
    out = np.zeros(N * st)
    flops = o.execute(u, out, d, st)
    assert flops == int(golden[key + "/flops"])
    assert relerr(out, golden[key + "/out"]) <= PORT_TOL


def test_nodal_plan_tables_bitwise(orc, golden):
    # barycentric leaf matrices T (leg2cheb.c:997-1031) and the two child
    # interpolation matrices B0 | B1 (leg2cheb.c:1076-1100)
    o = orc.Oracle(1024, 64, 2, lagrange=1)
    assert np.array_equal(o.T(), golden["nodal_plan_N1024_s64/T"])
    assert np.array_equal(o.B(), golden["nodal_plan_N1024_s64/B"])


@pytest.mark.parametrize("d", [0, 1])
def test_nodal_and_modal_agree(orc, d):
    # two discretisations of the same far field: equal to rounding
    N = 8192
    u = make_input(N, "sign", 9)
    a = orc.Oracle(N, 64, 2, lagrange=0)(u, d)[:N]
    b = orc.Oracle(N, 64, 2, lagrange=1)(u, d)[:N]
    assert relerr(b, a) <= 5e-15


def test_known_answers_N20(orc):
    # src/bin/l2c.c:69-74 (test_accuracy): first five outputs for an all-ones input
    a = [1.7913439415860921e00, 2.3408718378050253e00, 1.8833606631960720e00,
         1.6587642683880404e00, 1.4417173322290182e00]
    b = [5.2631578947368418e-01, 7.5187969924812026e-02, 1.3268465280849182e-01,
         1.7768205680441512e-01, 2.4367824933176932e-01]
    o = orc.Oracle(20, 64, 2)
    u = np.ones(20)
    l2c = o(u, 0)
    c2l = o(u, 1)
    assert np.sqrt(np.sum((l2c[:5] - a) ** 2)) < 1e-7
    assert np.sqrt(np.sum((c2l[:5] - b) ** 2)) < 1e-7
    assert np.max(np.abs(l2c[:5] - a)) < 1e-15 * 4
    assert np.max(np.abs(c2l[:5] - b)) < 1e-15


def test_lambda_known_values(orc):
    lib = orc.load()
    # src/bin/l2c.c:695-707
    z0 = [1.7724538509055161e00, 8.8622692545275805e-01, 6.6467019408956851e-01]
    for k in range(3):
        assert abs(lib.orc_Lambda(float(k)) - z0[k]) < 1e-15
    assert abs(lib.orc_Lambda(24.5) - 0.20100243720317808186742632) < 1e-17


def test_lambda_bitwise(orc, golden):
    lib = orc.load()
    z = golden["Lambda_z"]
    mine = np.array([lib.orc_Lambda(float(v)) for v in z])
    assert np.array_equal(mine, golden["Lambda"])
    mine = np.array([lib.orc_LambdaI(i) for i in range(256)])
    assert np.array_equal(mine, golden["LambdaI"])


def test_binomial_tables(orc, golden):
    lib = orc.load()
    o = orc.Oracle(512, 32, 2)
    B = np.ctypeslib.as_array(lib.orc_plan_B(o._p), (171,))
    BT = np.ctypeslib.as_array(lib.orc_plan_BT(o._p), (171,))
    assert np.array_equal(B, golden["BMe"])
    assert np.array_equal(BT, golden["BMeT"])


@pytest.mark.parametrize("N,maxs", [(512, 64), (512, 32), (1000, 36), (2048, 64), (4096, 32)])
@pytest.mark.parametrize("dist", ["uniform", "sign"])
def test_oracle_vs_extended_precision(orc, N, maxs, dist):
    u = make_input(N, dist, 42 + N)
    o = orc.Oracle(N, maxs, 2)
    assert direct_ld.rel_maxnorm(o(u, 0)[:N], direct_ld.l2c_direct(u)) < 5e-15
    assert direct_ld.rel_maxnorm(o(u, 1)[:N], direct_ld.c2l_direct(u)) < 5e-15


@pytest.mark.parametrize("seed", range(12))
def test_oracle_random_shapes_vs_extended_precision(orc, seed):
    """The checker itself on seeded random lengths (from 2, so the direct
    method too), leaf sizes and input distributions, against the
    extended-precision direct sums: at most 1.7e-15 measured, bar 5e-15."""
    rng = np.random.default_rng(6000 + seed)
    N = int(np.exp(rng.uniform(np.log(2), np.log(6000))))
    maxs = int(rng.integers(8, 65))
    u = make_input(N, ("uniform", "sign", "gauss")[seed % 3], seed)
    o = orc.Oracle(N, maxs, 2)
    assert direct_ld.rel_maxnorm(o(u, 0)[:N], direct_ld.l2c_direct(u)) < 5e-15, (N, maxs)
    assert direct_ld.rel_maxnorm(o(u, 1)[:N], direct_ld.c2l_direct(u)) < 5e-15, (N, maxs)


@pytest.mark.parametrize("N", [257, 1023, 4097])
def test_oracle_odd_N_l2c_vs_extended_precision(orc, N):
    # the reference itself cannot run these (leg2cheb.c:283-294 overruns for odd N)
    u = make_input(N, "uniform", N)
    o = orc.Oracle(N, 64, 2)
    assert direct_ld.rel_maxnorm(o(u, 0)[:N], direct_ld.l2c_direct(u)) < 5e-15


@pytest.mark.parametrize("N,maxs", [(512, 64), (512, 32)])
def test_roundtrip_matches_reference(orc, golden, N, maxs):
    # like `l2c -N512 -d2` (src/bin/l2c.c:10-65)
    u = make_input(N, "uniform", 7)
    o = orc.Oracle(N, maxs, 2)
    c = o(u, 0)
    b = o(c, 1)
    assert relerr(c, golden[f"roundtrip_{N}_{maxs}/cheb"]) < PORT_TOL
    assert relerr(b, golden[f"roundtrip_{N}_{maxs}/leg"]) < 1e-13
    assert relerr(b, u) < 1e-10  # the reference test's own bound (l2c.c:58-60)
