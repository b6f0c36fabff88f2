"""The mixed form (L2C_PLAN_MIXED): leaf, transfer and far-field products on
FP16 tensor cores from exact 9-bit digit slices of the FP64 operands, with
exact integer recombination.  Same
accuracy bar as the FP64 path: 1e-14 relative max-norm against the oracle,
per direction, on single vectors and on batches (where the far-field blocks
also run on the tensor cores)."""
import numpy as np
import pytest

from oracle import direct_ld
from tests.conftest import relerr
from tests.golden.cases import make_input

pytestmark = pytest.mark.gpu

TOL = 1e-14


@pytest.mark.parametrize("N,maxs", [(512, 64), (4096, 16), (4096, 32), (5000, 50), (65536, 16),
                                    (1 << 20, 32), (1 << 20, 64), (300, 18), (1495, 64),
                                    (1600, 64), (3000, 64)])
@pytest.mark.parametrize("dist", ["uniform", "sign"])
def test_mixed_single_vector(lib, orc, N, maxs, dist):
    u = make_input(N, dist, N + maxs)
    p = lib.Plan(N, maxs, mixed=True)
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        out = np.zeros(N)
        p.execute(u, out, d)
        assert relerr(out, o(u, d)[:N]) <= TOL, (N, maxs, d)


@pytest.mark.parametrize("N,maxs,count", [(1024, 64, 16), (1024, 16, 64), (16384, 16, 8),
                                          (2000, 50, 5), (1495, 64, 12), (1600, 64, 6)])
def test_mixed_batch(lib, orc, N, maxs, count):
    x = make_input(N * count, "gauss", 3).reshape(count, N) / (np.arange(N) + 1.0)
    x = np.ascontiguousarray(x)
    p = lib.Plan(N, maxs, mixed=True)
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        out = np.zeros_like(x)
        p.execute_batched(x, out, d, count, N, 1)
        for i in (0, count // 2, count - 1):
            assert relerr(out[i], o(x[i], d)[:N]) <= TOL, (i, d)


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("N,maxs,count", [(6902, 16, 4), (7000, 16, 1), (2100, 16, 3),
                                          (6902, 32, 2)])
def test_batch_gaps_untouched(lib, orc, mixed, N, maxs, count):
    """Vectors dist > N apart: the gaps between them keep their contents.  With
    N < Nn - 2h the last leaf targets cover outputs past N (K h > N); nothing
    may be read or written there (N = 6902, s = 14: K h = 7112).  The outputs
    themselves start at zero: like the reference's execute, the transform adds
    to the output array."""
    dist = N + 300
    x = np.full((count, dist), np.nan)
    x[:, :N] = make_input(count * N, "gauss", 11).reshape(count, N)
    p = lib.Plan(N, maxs, mixed=mixed)
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        out = np.full((count, dist), 12345.0)
        out[:, :N] = 0.0
        p.execute_batched(x, out, d, count, dist, 1)
        assert np.all(out[:, N:] == 12345.0), (N, d)
        for v in range(count):
            assert relerr(out[v, :N], o(x[v, :N], d)[:N]) <= TOL, (N, maxs, d, v)


def test_mixed_vs_extended_precision(lib):
    N = 8192
    u = make_input(N, "uniform", 77)
    p = lib.Plan(N, 16, mixed=True)
    for d, f in ((0, direct_ld.l2c_direct), (1, direct_ld.c2l_direct)):
        out = np.zeros(N)
        p.execute(u, out, d)
        assert direct_ld.rel_maxnorm(out, f(u)) < 5e-15


def test_mixed_wide_dynamic_range(lib, orc):
    # per-column scaling must cope with inputs spanning many orders of magnitude
    N = 16384
    rng = np.random.default_rng(5)
    u = rng.standard_normal(N) * 10.0 ** rng.uniform(-12, 12, N)
    p = lib.Plan(N, 32, mixed=True)
    o = orc.Oracle(N, 32, 2)
    for d in (0, 1):
        out = np.zeros(N)
        p.execute(u, out, d)
        assert relerr(out, o(u, d)[:N]) <= TOL


def test_mixed_rejects_large_leaves(lib):
    with pytest.raises(lib.L2CError, match="s <= 64"):
        lib.Plan(1 << 16, 200, mixed=True)  # s = 128


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("count", [1, 16, 64])
def test_launch_options_bitwise(lib, monkeypatch, mixed, count):
    """Programmatic dependent launch, the band on the second stream, graph
    replay, the tile buffer depth, the chain's scheduling priority and the
    band's CTA size, vectors per thread, grid cap, weight table and fork point,
    and (mixed form) the coarsest transfer levels in one launch or one launch
    per level and the finest levels' far field on a third stream, change only
    when work runs, never what it computes: every
    setting gives the same bits as the default plan (count = 64: the band as
    dense register tiles, with its table or weights formed on the fly)."""
    N = 16384
    x = np.ascontiguousarray(make_input(N * count, "gauss", 11).reshape(count, N))

    def run():
        p = lib.Plan(N, 16, mixed=mixed)
        outs = []
        for d in (0, 1):
            out = np.zeros_like(x)
            for _ in range(2):  # capture, then replay
                out[:] = 0
                p.execute_batched(x, out, d, count, N, 1)
            outs.append(out)
        p.close()
        return outs

    want = run()
    for env in ({"L2C_PDL": "0"}, {"L2C_PDL": "7"}, {"L2C_PDL": "7", "L2C_OVERLAP": "0"},
                {"L2C_PDL": "7", "L2C_OVERLAP": "1"}, {"L2C_PDL": "7", "L2C_NO_GRAPHS": "1"},
                {"L2C_MZ_NBUF": "2"}, {"L2C_CHAIN_PRIO": "0"}, {"L2C_CHAIN_PRIO": "1"},
                # the band's launch choices (the autotuner searches these too)
                {"L2C_NEAR_VB": "1"}, {"L2C_NEAR_VB": "2"}, {"L2C_NEAR_VB": "4"},
                {"L2C_NEAR_THREADS": "256"}, {"L2C_NEAR_CTAS": "456"},
                {"L2C_NEAR_THREADS": "256", "L2C_NEAR_VB": "2", "L2C_NEAR_CTAS": "912"},
                {"L2C_NEAR_TABLE": "0"}, {"L2C_NEAR_TABLE": "1"},
                {"L2C_BAND_FORK": "1"}, {"L2C_BAND_FORK": "2"}, {"L2C_BAND_FORK": "3"},
                {"L2C_BAND_FORK": "2", "L2C_PDL": "7"},
                # the mixed form's coarsest transfer levels one launch each
                {"L2C_MZ_TOP": "0"}, {"L2C_MZ_TOP": "0", "L2C_PDL": "0"},
                # the per-level structure the autotuner searches
                {"L2C_MZ_TOP_LVL": "5"}, {"L2C_MZ_TOP_LVL": "3", "L2C_MZ_TOP_G": "1"},
                {"L2C_MZ_TOP_G": "4"}, {"L2C_TREE_L0": "1"}, {"L2C_TREE_L0": "3"},
                {"L2C_BAND_BSEG": "1"}, {"L2C_BAND_BSEG": "4"},
                # the finest levels' far field on a third stream (none, 1 .. 4
                # levels), also without graphs and with the top launch off
                {"L2C_FAR_SPLIT": "0"}, {"L2C_FAR_SPLIT": "1"}, {"L2C_FAR_SPLIT": "3"},
                {"L2C_FAR_SPLIT": "4"}, {"L2C_FAR_SPLIT": "3", "L2C_NO_GRAPHS": "1"},
                {"L2C_FAR_SPLIT": "3", "L2C_MZ_TOP": "0"},
                {"L2C_FAR_SPLIT": "2", "L2C_MZ_TOP_LVL": "5", "L2C_BAND_FORK": "3"},
                # the tiled band's thin variant (one vector per lane)
                {"L2C_BAND_THIN": "1"}, {"L2C_BAND_THIN": "1", "L2C_NEAR_TABLE": "0"},
                {"L2C_BAND_THIN": "1", "L2C_NEAR_CTAS": "608"},
                # the far field on the fifth-generation tensor cores
                {"L2C_FAR_TC": "1"}, {"L2C_FAR_TC": "1", "L2C_FAR_SPLIT": "0"},
                {"L2C_FAR_TC": "1", "L2C_PDL": "7"}, {"L2C_FAR_TC": "1", "L2C_NO_GRAPHS": "1"},
                # the far field's columns per CTA (one or two tiles per warp)
                {"L2C_FAR_COLS": "64"}, {"L2C_FAR_COLS": "128"},
                {"L2C_FAR_COLS": "64", "L2C_FAR_SPLIT": "0"},
                # the tensor-core band's 16-vector tiles per warp
                {"L2C_MZ_BAND_TPW": "2"}, {"L2C_MZ_BAND_TPW": "4"}):
        with monkeypatch.context() as m:
            for k, v in env.items():
                m.setenv(k, v)
            got = run()
        for d in (0, 1):
            assert np.array_equal(got[d], want[d]), (env, d)


@pytest.mark.parametrize("N,maxs,count", [(2000, 16, 65), (4096, 32, 100), (1024, 64, 96),
                                          (5000, 50, 8), (16384, 16, 256)])
def test_far_tc_bitwise(lib, orc, monkeypatch, N, maxs, count):
    """The far field on the fifth-generation tensor cores (L2C_FAR_TC=1:
    tcgen05 products with the diagonal sums in tensor memory, k_mz_far_tc)
    forms the same integers as the mma.sync far field, so every output has the
    same bits; column chunks past 128 columns and a partly filled last chunk
    (count 65, 100), leaf sizes 16 .. 64, and the 256 x 16384 batch.  Some
    vectors are also checked against the oracle."""
    x = np.ascontiguousarray(make_input(N * count, "gauss", 3 + count).reshape(count, N))

    def run():
        p = lib.Plan(N, maxs, mixed=True)
        outs = []
        for d in (0, 1):
            out = np.zeros_like(x)
            p.execute_batched(x, out, d, count, N, 1)
            outs.append(out)
        p.close()
        return outs

    want = run()
    with monkeypatch.context() as m:
        m.setenv("L2C_FAR_TC", "1")
        got = run()
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        assert np.array_equal(got[d], want[d]), d
        for v in (0, count // 2, count - 1):
            assert relerr(got[d][v], o(x[v], d)[:N]) <= TOL, (d, v)


@pytest.mark.parametrize("N,maxs,count,dist", [(16384, 16, 256, "gauss"), (4096, 16, 70, "uniform"),
                                               (1000, 16, 64, "gauss"), (20000, 16, 100, "sign"),
                                               (16384, 32, 256, "gauss"), (8192, 32, 65, "uniform"),
                                               (3000, 32, 64, "sign")])
def test_mixed_band_forms(lib, orc, monkeypatch, N, maxs, count, dist):
    """Batches at s = 16 and s = 32 run the near-field band of the full blocks
    on the tensor cores (k_mz_band, k_mz_band2: exact integer products of the
    split weights and windows, one rounding) and the last block in FP64;
    L2C_MZ_BAND=0 keeps the FP64 tiled band.  Both agree with the oracle to
    1e-14 on every vector."""
    x = np.ascontiguousarray(make_input(N * count, dist, 9 + count).reshape(count, N))
    o = orc.Oracle(N, maxs, 2)
    want = [np.stack([o(x[v], d)[:N] for v in range(count)]) for d in (0, 1)]
    for env in ("1", "0"):
        with monkeypatch.context() as m:
            m.setenv("L2C_MZ_BAND", env)
            p = lib.Plan(N, maxs, mixed=True)
            for d in (0, 1):
                out = np.zeros_like(x)
                p.execute_batched(x, out, d, count, N, 1)
                for v in range(count):
                    assert relerr(out[v], want[d][v]) <= TOL, (env, d, v)
            p.close()


@pytest.mark.parametrize("count", [65, 100])
def test_mixed_far_column_chunks(lib, orc, count):
    """Batches past one far-field CTA's 128 columns (2 parities x count): the
    column chunks along the grid's y, the last one partly filled."""
    N, maxs = 2000, 16
    x = np.ascontiguousarray(make_input(N * count, "gauss", count).reshape(count, N))
    p = lib.Plan(N, maxs, mixed=True)
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        out = np.zeros_like(x)
        p.execute_batched(x, out, d, count, N, 1)
        for v in range(count):
            assert relerr(out[v], o(x[v], d)[:N]) <= TOL, (count, d, v)


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_non_finite_inputs(lib, orc, bad):
    """Inf and NaN inputs.  The plain form gives the oracle's pattern of
    non-finite outputs exactly (they spread through the same sums).  The mixed
    form's fixed-point far field cannot carry them: a vector holding one gets
    non-finite outputs wherever the oracle does (and more), and the other
    vectors of the batch keep their bits."""
    N, maxs, count = 4096, 16, 6
    x = np.ascontiguousarray(make_input(N * count, "gauss", 21).reshape(count, N))
    xb = x.copy()
    xb[2, 1500] = bad
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        want = ~np.isfinite(o(xb[2], d)[:N])
        assert want.any()
        p = lib.Plan(N, maxs)
        out = np.zeros_like(xb)
        p.execute_batched(xb, out, d, count, N, 1)
        assert np.array_equal(~np.isfinite(out[2]), want), d
        q = lib.Plan(N, maxs, mixed=True)
        clean, got = np.zeros_like(x), np.zeros_like(xb)
        q.execute_batched(x, clean, d, count, N, 1)
        q.execute_batched(xb, got, d, count, N, 1)
        assert np.all(~np.isfinite(got[2]) >= want), d
        for v in (0, 1, 3, 4, 5):
            assert np.array_equal(got[v], clean[v]), (d, v)


@pytest.mark.parametrize("N,maxs,count", [(16384, 16, 64), (16384, 16, 100), (4096, 32, 70),
                                          (1024, 64, 96), (6000, 24, 65), (20000, 40, 64)])
def test_band_tiles_vs_oracle(lib, orc, monkeypatch, N, maxs, count):
    """Batches of 64 and more vectors take the band as dense register tiles
    (full blocks) plus the per-output kernel (last block); chunks of 64 or 32
    vectors, the last one partly filled.  Every vector against the oracle, and
    the same batch with the tiles switched off (L2C_BAND_TILE=0) within the
    same bar."""
    x = np.ascontiguousarray(make_input(N * count, "gauss", count + N).reshape(count, N))
    o = orc.Oracle(N, maxs, 2)
    outs = {}
    for env in ("1", "0"):
        with monkeypatch.context() as m:
            m.setenv("L2C_BAND_TILE", env)
            p = lib.Plan(N, maxs)
        for d in (0, 1):
            out = np.zeros_like(x)
            p.execute_batched(x, out, d, count, N, 1)
            outs[env, d] = out
        p.close()
    for d in (0, 1):
        want = np.zeros_like(x)
        o.execute_batch(x, want, d, count, N)
        for v in range(count):
            assert relerr(outs["1", d][v], want[v]) <= TOL, (d, v)
            assert relerr(outs["1", d][v], outs["0", d][v]) <= TOL, (d, v)
