"""GPU parity: the CUDA path (through the C ABI) against the reference.

Tolerance: 1e-14 relative max-norm, max|y - y_ref| / max|y_ref|, per direction
(the FP64 bar of the transform's specification).  References:
  * golden vectors from the unmodified reference (tests/golden),
  * the oracle port (oracle/l2c_oracle.c) for cases the reference cannot run
    (odd-N L2C) or that are too big for fixtures,
  * the extended-precision direct sum (oracle/direct_ld.py)."""
import numpy as np
import pytest

from oracle import direct_ld
from tests.conftest import relerr
from tests.golden.cases import CASES, make_input

pytestmark = pytest.mark.gpu

TOL = 1e-14


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    return torch


@pytest.mark.parametrize("key", sorted(CASES))
def test_golden_cases_host_pointers(lib, golden, key):
    N, maxs, d, st, dist, seed = CASES[key]
    u = make_input(N * st, dist, seed)
    out = np.zeros(N * st)
    if key.startswith("direct"):
        p = lib.DirectPlan(N, 2)
        flops = p(u, out, d, st)
    else:
        p = lib.Plan(N, maxs, direction=2)
        flops = p.execute(u, out, d, st)
    assert flops == int(golden[key + "/flops"])
    assert relerr(out, golden[key + "/out"]) <= TOL


@pytest.mark.parametrize("key", [k for k in sorted(CASES) if k.startswith("ones_")])
def test_known_answers_N20(lib, key):
    # src/bin/l2c.c:69-74
    a = [1.7913439415860921e00, 2.3408718378050253e00, 1.8833606631960720e00,
         1.6587642683880404e00, 1.4417173322290182e00]
    b = [5.2631578947368418e-01, 7.5187969924812026e-02, 1.3268465280849182e-01,
         1.7768205680441512e-01, 2.4367824933176932e-01]
    d = 0 if "_d0_" in key else 1
    p = lib.Plan(20, 64)
    out = np.zeros(20)
    p.execute(np.ones(20), out, d)
    want = a if d == 0 else b
    assert np.sqrt(np.sum((out[:5] - want) ** 2)) < 1e-7
    assert np.max(np.abs(out[:5] - want)) < 4e-15


@pytest.mark.parametrize("N,maxs", [(512, 64), (4096, 32), (16384, 64), (1 << 18, 64)])
def test_plan_tables_match_oracle(lib, orc, N, maxs):
    p = lib.Plan(N, maxs)
    o = orc.Oracle(N, maxs, 2)
    # Lambda table: identical arithmetic on both sides
    assert np.array_equal(p.copy_table(2), o.lambda_table())
    assert np.array_equal(p.copy_table(5), o.T())
    for d in (0, 1):
        A = p.copy_table(d).reshape(-1, 18, 18)
        B = o.A(d).reshape(-1, 18, 18)
        err = np.max(np.abs(A - B), axis=(1, 2)) / np.max(np.abs(B), axis=(1, 2))
        assert err.max() < 1e-14


@pytest.mark.parametrize("N", [257, 1023, 4097, 20001])
def test_odd_N_l2c(lib, orc, N):
    # the reference overruns its arrays here (leg2cheb.c:283-294); the oracle port
    # and the extended-precision sum give the intended values
    u = make_input(N, "uniform", N)
    p = lib.Plan(N, 64)
    out = np.zeros(N)
    p.execute(u, out, 0)
    assert relerr(out, orc.Oracle(N, 64, 2)(u, 0)[:N]) <= TOL
    if N <= 5000:
        assert direct_ld.rel_maxnorm(out, direct_ld.l2c_direct(u)) < 5e-15


@pytest.mark.parametrize("N,maxs", [(1 << 20, 64), (1 << 20, 32), (1 << 21, 64), (1000003, 64)])
@pytest.mark.parametrize("d", [0, 1])
def test_large_single_vector_vs_oracle(lib, orc, N, maxs, d):
    u = make_input(N, "sign", 17 + d)
    if d == 0 and N % 2 == 1:
        u = u.copy()
    p = lib.Plan(N, maxs)
    out = np.zeros(N)
    flops = p.execute(u, out, d)
    want = orc.Oracle(N, maxs, 2)(u, d)[:N]
    assert relerr(out, want) <= TOL
    assert flops == p.flops(d)


@pytest.mark.parametrize("N", [1 << 20])
def test_vs_extended_precision_sample(lib, N):
    """Spot-check rows of a 2^20 transform against the extended-precision sum of
    those rows (cost O(N) per row)."""
    u = make_input(N, "sign", 99)
    p = lib.Plan(N, 64)
    out = np.zeros(N)
    p.execute(u, out, 0)
    a = direct_ld.lambda_table(N)
    ul = u.astype(np.longdouble)
    rows = [0, 1, 2, 777, N // 3, N // 2 + 1, N - 300, N - 2, N - 1]
    for i in rows:
        k = np.arange(0, (N - 1 - i) // 2 + 1)
        val = np.sum(a[k] * a[k + i] * ul[i + 2 * k]) * 2 / direct_ld._PI
        if i == 0:
            val /= 2
        assert abs(out[i] - float(val)) <= 2e-15 * np.max(np.abs(out))


def test_device_pointers_match_host_path(lib, torch_cuda):
    torch = torch_cuda
    N = 1 << 16
    u = make_input(N, "uniform", 5)
    p = lib.Plan(N, 64)
    for d in (0, 1):
        host = np.zeros(N)
        p.execute(u, host, d)
        du = torch.from_numpy(u).cuda()
        dout = torch.zeros(N, dtype=torch.float64, device="cuda")
        p.execute(du, dout, d)
        assert np.array_equal(dout.cpu().numpy(), host)


def test_accumulates_into_output_like_reference(lib, orc):
    # execute computes out = scale * (out_in + far + near) (leg2cheb.c:360-374, 519-532)
    N = 4096
    u = make_input(N, "uniform", 8)
    pre = make_input(N, "gauss", 9)
    p = lib.Plan(N, 64)
    o = orc.Oracle(N, 64, 2)
    for d in (0, 1):
        out = pre.copy()
        p.execute(u, out, d)
        want = pre.copy()
        o.execute(u, want, d)
        assert relerr(out, want) <= TOL


def test_batched_lines_of_3d_array(lib, orc):
    # lines along the last axis of a 64x64x1024 array; a 8x8x1024 slab here
    n0, n1, N = 8, 8, 1024
    x = make_input(n0 * n1 * N, "gauss", 3).reshape(n0, n1, N) / (np.arange(N) + 1.0) ** 2
    x = np.ascontiguousarray(x)
    p = lib.Plan(N, 64)
    o = orc.Oracle(N, 64, 2)
    for d in (0, 1):
        out = np.zeros_like(x)
        flops = p.execute_batched(x, out, d, n0 * n1, N, 1)
        assert flops == n0 * n1 * p.flops(d)
        for i in (0, 17, 63):
            line = x.reshape(-1, N)[i]
            assert relerr(out.reshape(-1, N)[i], o(line, d)[:N]) <= TOL


def test_batched_strided_axis0(lib, orc):
    # lines along axis 0 of a (N, n1) array: dist = 1, stride = n1
    N, n1 = 1000, 37
    x = np.ascontiguousarray(make_input(N * n1, "uniform", 4).reshape(N, n1))
    p = lib.Plan(N, 36)
    o = orc.Oracle(N, 36, 2)
    for d in (0, 1):
        out = np.zeros_like(x)
        p.execute_batched(x, out, d, n1, 1, n1)
        for j in (0, 5, 36):
            assert relerr(out[:, j], o(np.ascontiguousarray(x[:, j]), d)[:N]) <= TOL


@pytest.mark.parametrize("axis", [0, 1, -1])
def test_execute2d_matches_lines(lib, orc, axis):
    # src/bin/l2c.c:297-351 (test_forward_2d) and 353-393 (round trip)
    N0, N1 = 400, 402
    x = np.ascontiguousarray(make_input(N0 * N1, "uniform", 12).reshape(N0, N1))
    p2 = lib.Plan2D(N0, N1, axis, maxs=36)
    out = np.zeros_like(x)
    p2(x, out, 0)
    o0, o1 = orc.Oracle(N0, 36, 2), orc.Oracle(N1, 36, 2)
    if axis == 0:
        want = np.stack([o0(np.ascontiguousarray(x[:, j]), 0)[:N0] for j in range(N1)], axis=1)
    elif axis == 1:
        want = np.stack([o1(x[i], 0)[:N1] for i in range(N0)])
    else:
        t = np.stack([o0(np.ascontiguousarray(x[:, j]), 0)[:N0] for j in range(N1)], axis=1)
        want = np.stack([o1(np.ascontiguousarray(t[i]), 0)[:N1] for i in range(N0)])
    assert relerr(out, want) <= 1e-13 if axis == -1 else relerr(out, want) <= TOL
    if axis == -1:
        back = np.zeros_like(x)
        p2(out, back, 1)
        assert np.sqrt(np.sum((back - x) ** 2)) < 1e-8  # src/bin/l2c.c:386-388


@pytest.mark.parametrize("N0,N1", [(5, 7), (30, 11), (64, 200)])
def test_execute2d_direct_columns_like_reference(lib, orc, N0, N1):
    """Columns short enough for the direct path (L = 0): the reference's
    execute2D calls execute() per column with stride N1 (leg2cheb.c:1270-1274),
    and each call zeroes [0, N0) and reads its L2C input contiguously from the
    column's start, reaching the neighbouring columns.  The result is that of
    the calls in order, every time (graph capture, then replay)."""
    x = np.ascontiguousarray(make_input(N0 * N1, "gauss", N0).reshape(N0, N1))
    p2 = lib.Plan2D(N0, N1, 0, maxs=64)
    o = orc.Oracle(N0, 64, 2)
    assert o.L == 0
    for d in (0, 1):
        xf, wf = x.ravel(), np.zeros(N0 * N1)
        for j in range(N1):
            o.execute(xf[j:], wf[j:], d, N1)
        for _ in range(3):
            out = np.zeros_like(x)
            p2(x, out, d)
            assert relerr(out.ravel(), wf) <= TOL, d


def test_directM_directL_match_oracle_near_field(lib, orc):
    # near field + final scaling only (leg2cheb.c:236-376, 378-535)
    for N, st in ((2048, 1), (1000, 3)):
        u = make_input(N * st, "uniform", 21)
        p = lib.Plan(N, 64 if N == 2048 else 36)
        o = orc.Oracle(N, 64 if N == 2048 else 36, 2)
        out, want = np.zeros(N * st), np.zeros(N * st)
        fm = p.directM(u, out, st)
        assert fm == o.directM(u, want, st)
        assert relerr(out, want) <= TOL
        # directL takes the premultiplied contiguous input
        v = u[: N * st : st] * np.arange(N)
        v[:2] = u[: 2 * st : st]
        v = np.ascontiguousarray(v)
        out, want = np.zeros(N * st), np.zeros(N * st)
        fl = p.directL(v, out, st)
        assert fl == o.directL(v, want, st)
        assert relerr(out, want) <= TOL


def test_unplanned_direction_fails_cleanly(lib):
    p = lib.Plan(4096, 64, direction=0)
    out = np.zeros(4096)
    with pytest.raises(lib.L2CError, match="not planned"):
        p.execute(np.ones(4096), out, 1)
    with pytest.raises(lib.L2CError):
        p.execute(np.ones(4096), out, 3)


def test_repeatable_bitwise(lib):
    N = 1 << 18
    u = make_input(N, "gauss", 1)
    p = lib.Plan(N, 64)
    r = []
    for _ in range(3):
        out = np.zeros(N)
        p.execute(u, out, 0)
        r.append(out)
    assert np.array_equal(r[0], r[1]) and np.array_equal(r[1], r[2])


@pytest.mark.parametrize("N", [1 << 22])
def test_full_size_properties(lib, N):
    """N = 2^22 (the mixed-precision single-vector size): linearity and the
    L2C -> C2L round trip, size-independent properties of the exact transform."""
    p = lib.Plan(N, 64)
    u = make_input(N, "sign", 3)
    v = make_input(N, "gauss", 4) / (np.arange(N) + 1.0)
    fu, fv, fw = np.zeros(N), np.zeros(N), np.zeros(N)
    p.execute(u, fu, 0)
    p.execute(v, fv, 0)
    p.execute(2.0 * u - 0.5 * v, fw, 0)
    assert relerr(fw, 2.0 * fu - 0.5 * fv) < 1e-14
    back = np.zeros(N)
    p.execute(fu, back, 1)
    assert relerr(back, u) < 1e-12


@pytest.mark.parametrize("N,maxs", [(4096, 64), (5001, 64), (1 << 20, 32), (300, 64),
                                    ((1 << 20) + 1, 64), (200000, 50)])
def test_precomputed_band_weights_bitwise(lib, N, maxs):
    # create_fmm's precompute = 1 keeps the band weights in device memory; the
    # weights are the same products, so results are bit-identical (odd leaf
    # sizes too: s = 33 and 49 with the register-window band, whose table rows
    # are then not 16-byte aligned)
    u = make_input(N, "uniform", N + 1)
    p0 = lib.Plan(N, maxs)
    p1 = lib.Plan(N, maxs, precompute=1)
    for d in (0, 1):
        o0, o1 = np.zeros(N), np.zeros(N)
        p0.execute(u, o0, d)
        p1.execute(u, o1, d)
        assert np.array_equal(o0, o1)


def test_graph_cache_across_shapes(lib, orc):
    # captured launch sequences are cached per call shape; growing the scratch
    # buffers must invalidate them
    N = 1024
    p = lib.Plan(N, 64)
    o = orc.Oracle(N, 64, 2)
    rng = np.random.default_rng(0)
    for count in (1, 4, 1, 64, 4, 1, 256, 64):
        x = rng.uniform(-1, 1, (count, N))
        for d in (0, 1):
            out = np.zeros_like(x)
            p.execute_batched(x, out, d, count, N, 1)
            for i in {0, count - 1}:
                assert relerr(out[i], o(x[i], d)[:N]) <= TOL


def test_async_device_execution(lib, orc, torch_cuda):
    torch = torch_cuda
    N, count = 16384, 8
    x = make_input(N * count, "sign", 5).reshape(count, N)
    p = lib.Plan(N, 64)
    dx = torch.from_numpy(x).cuda()
    outs = [torch.zeros_like(dx) for _ in range(3)]
    for o_ in outs:
        p.execute_async(dx, o_, 0, count, N, 1)
    p.synchronize()
    o = orc.Oracle(N, 64, 2)
    want = o(x[3], 0)[:N]
    for o_ in outs:
        assert relerr(o_.cpu().numpy()[3], want) <= TOL


def ragged_lengths(count, seed, lo=64, hi=65536):
    """N log-uniform in [lo, hi] (the ragged-list workload's distribution)."""
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(np.int64)


@pytest.mark.parametrize("maxs", [64, 36])
def test_ragged_batch_matches_per_vector(lib, orc, maxs):
    Ns = list(ragged_lengths(40, 7, 20, 20000)) + [20, 255, 256, 257, 300, 1023, 5001]
    p = lib.RaggedPlan(Ns, maxs)
    u = make_input(p.total, "uniform", 3)
    for d in (0, 1):
        out = np.zeros(p.total)
        flops = p(u, out, d)
        want_flops = 0
        for v, N in enumerate(Ns):
            a, b = p.offsets[v], p.offsets[v + 1]
            o = orc.Oracle(int(N), maxs, 2)
            w = np.zeros(int(N))
            want_flops += o.execute(np.ascontiguousarray(u[a:b]), w, d)
            assert relerr(out[a:b], w) <= TOL, (v, N, d)
        assert flops == want_flops


def test_ragged_accumulates_like_execute(lib):
    Ns = [100, 4096, 777, 65536, 3000]
    p = lib.RaggedPlan(Ns, 64)
    u = make_input(p.total, "sign", 1)
    pre = make_input(p.total, "gauss", 2)
    for d in (0, 1):
        out = pre.copy()
        p(u, out, d)
        for v, N in enumerate(Ns):
            a, b = p.offsets[v], p.offsets[v + 1]
            single = lib.Plan(int(N), 64)
            want = pre[a:b].copy()
            single.execute(np.ascontiguousarray(u[a:b]), want, d)
            assert relerr(out[a:b], want) <= TOL


def test_ragged_device_pointers_and_launch_count(lib, torch_cuda):
    torch = torch_cuda
    Ns = ragged_lengths(500, 11)
    p = lib.RaggedPlan(Ns, 64)
    u = make_input(p.total, "uniform", 4)
    host = np.zeros(p.total)
    p(u, host, 1)
    du = torch.from_numpy(u).cuda()
    dout = torch.zeros_like(du)
    before = p.launch_count()
    p.execute_async(du, dout, 1)
    p.synchronize()
    assert p.launch_count() - before <= 24  # independent of the 500 vectors
    assert np.array_equal(dout.cpu().numpy(), host)


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("count,N,stride", [(1, 1 << 16, 1), (1, 4097, 3), (16, 4096, 1)])
def test_pinned_host_buffers_in_place(lib, torch_cuda, monkeypatch, mixed, count, N, stride):
    """Page-locked host buffers are read and written in place through their
    device mapping (no staging copies); results are the staged path's bits."""
    torch = torch_cuda
    maxs = 16 if mixed else 64
    if mixed and stride != 1:
        pytest.skip("strided lines are covered by the plain form")
    dist = N * stride
    x = make_input(count * dist, "sign", N + count)
    want = []
    with monkeypatch.context() as m:
        m.setenv("L2C_ZERO_COPY", "0")
        p = lib.Plan(N, maxs, mixed=mixed)
        for d in (0, 1):
            out = np.zeros(count * dist)
            p.execute_batched(x, out, d, count, dist, stride)
            want.append(out)
        p.close()
    p = lib.Plan(N, maxs, mixed=mixed)
    hx = torch.from_numpy(x).pin_memory()
    for d in (0, 1):
        ho = torch.zeros(count * dist, dtype=torch.float64).pin_memory()
        for _ in range(2):  # capture, then replay
            ho.zero_()
            p.execute_batched(hx, ho, d, count, dist, stride)
        assert np.array_equal(ho.numpy(), want[d]), d


def test_dlpack_device_arrays(lib, torch_cuda):
    """Any DLPack producer is accepted in place (here a minimal one that
    exports a CUDA tensor only through __dlpack__)."""
    torch = torch_cuda

    class Producer:
        def __init__(self, t):
            self._t = t

        def __dlpack__(self, **kw):
            return self._t.__dlpack__(**kw)

        def __dlpack_device__(self):
            return self._t.__dlpack_device__()

    N = 4096
    u = make_input(N, "sign", 3)
    p = lib.Plan(N, 64)
    want = np.zeros(N)
    p.execute(u, want, 0)
    du = torch.from_numpy(u).cuda()
    dout = torch.zeros(N, dtype=torch.float64, device="cuda")
    p.execute(Producer(du), Producer(dout), 0)
    assert np.array_equal(dout.cpu().numpy(), want)


@pytest.mark.parametrize("N", [1, 2, 3, 5, 8])
def test_tiny_lengths_match_oracle(lib, orc, N):
    # the direct path at the smallest lengths, both directions, strides 1 and 2
    u = make_input(2 * N, "uniform", 40 + N)
    p = lib.Plan(N, 64)
    o = orc.Oracle(N, 64, 2)
    for d in (0, 1):
        for st in (1, 2):
            out = np.zeros(2 * N)
            want = np.zeros(2 * N)
            assert p.execute(u, out, d, st) == o.execute(u, want, d, st)
            assert relerr(out, want) <= TOL


def test_empty_length_is_refused(lib):
    with pytest.raises(lib.L2CError, match="positive"):
        lib.Plan(0, 64)


@pytest.mark.parametrize("seed", range(12))
def test_random_shapes_vs_oracle(lib, orc, seed):
    """Seeded random lengths, leaf sizes, strides and batch counts, both
    directions and both discretisations (modal, nodal), against the oracle at
    the 1e-14 bar."""
    rng = np.random.default_rng(1000 + seed)
    N = int(np.exp(rng.uniform(np.log(20), np.log(70000))))
    maxs = int(rng.choice([18, 32, 36, 50, 64, 100]))
    stride = int(rng.choice([1, 1, 2, 3]))
    count = int(rng.choice([1, 2, 5]))
    lagrange = int(rng.integers(0, 2))
    dist = N * stride + int(rng.integers(0, 3))
    x = make_input(count * dist, "uniform", seed)
    p = lib.Plan(N, maxs, lagrange=lagrange)
    o = orc.Oracle(N, maxs, 2, lagrange=lagrange)
    for d in (0, 1):
        out = np.zeros(count * dist + 1)
        p.execute_batched(x, out, d, count, dist, stride)
        for v in range(count):
            want = np.zeros(dist + 1)
            o.execute(np.ascontiguousarray(x[v * dist:(v + 1) * dist]), want, d, stride)
            got = out[v * dist:v * dist + (N - 1) * stride + 1:stride]
            ref = want[:(N - 1) * stride + 1:stride]
            assert relerr(got, ref) <= TOL, (N, maxs, stride, count, lagrange, d, v)


@pytest.mark.parametrize("seed", range(8))
def test_random_shapes_mixed_vs_oracle(lib, orc, seed):
    """The mixed form on seeded random shapes (leaf sizes s <= 64, batches of
    1 to 12 vectors: below and above the tensor-core far-field threshold)."""
    rng = np.random.default_rng(2000 + seed)
    N = int(np.exp(rng.uniform(np.log(300), np.log(70000))))
    maxs = int(rng.choice([16, 24, 32, 64]))
    count = int(rng.choice([1, 3, 4, 12]))
    x = np.ascontiguousarray(make_input(count * N, "gauss", seed).reshape(count, N))
    p = lib.Plan(N, maxs, mixed=True)
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        out = np.zeros_like(x)
        p.execute_batched(x, out, d, count, N, 1)
        for v in range(count):
            assert relerr(out[v], o(x[v], d)[:N]) <= TOL, (N, maxs, count, d, v)


@pytest.mark.parametrize("seed", range(24))
def test_random_layouts_whole_buffer(lib, orc, seed):
    """Every form (modal, nodal, mixed) on a seeded random shape and layout
    (N from 2, so the direct path too; any maxs in [8, 64]; strides 1-3;
    vectors dist >= (N-1) stride + 1 apart with random padding), compared over
    the WHOLE buffer with the oracle run on an identical buffer: the outputs
    at j stride to 1e-14, every other position exactly (untouched, or zeroed
    where the reference's direct path zeroes [0, N) contiguously).  With
    L >= 1 the input's gaps hold NaN, so a read there would show."""
    form, N, maxs, stride, count, dist = random_layout(seed)
    lagrange = 1 if form == "nodal" else 0
    p = lib.Plan(N, maxs, lagrange=lagrange, mixed=form == "mixed")
    o = orc.Oracle(N, maxs, 2, lagrange=lagrange)
    pos = np.zeros(count * dist + 7, dtype=bool)  # the transform's own positions
    for v in range(count):
        pos[v * dist:v * dist + (N - 1) * stride + 1:stride] = True
    x = np.full(pos.size, np.nan if p.L >= 1 else 3.0)
    x[pos] = make_input(int(pos.sum()), "gauss", seed)
    for d in (0, 1):
        out0 = np.full(pos.size, 7.0)
        out0[pos] = 0.0
        got = out0.copy()
        p.execute_batched(x, got, d, count, dist, stride)
        want = out0.copy()
        for v in range(count):
            seg = slice(v * dist, v * dist + dist)
            w = np.ascontiguousarray(want[seg])
            o.execute(np.ascontiguousarray(x[seg]), w, d, stride)
            want[seg] = w
        why = (form, N, maxs, stride, count, dist, d)
        assert np.array_equal(got[~pos], want[~pos]), why
        assert relerr(got[pos], want[pos]) <= TOL, why


@pytest.mark.parametrize("seed", range(6))
def test_random_ragged_vs_oracle(lib, orc, seed):
    """Seeded random ragged lists (1 to 60 vectors, N log-uniform from 1 to
    70000, so direct-path vectors too; any maxs in [8, 64]) on nonzero
    incoming outputs, against the oracle per vector; the slots past the last
    vector keep their contents."""
    rng = np.random.default_rng(4000 + seed)
    count = int(rng.integers(1, 61))
    Ns = [int(n) for n in np.exp(rng.uniform(0, np.log(70000), count))]
    maxs = int(rng.integers(8, 65))
    p = lib.RaggedPlan(Ns, maxs)
    u = make_input(p.total, "gauss", seed)
    pre = np.concatenate([make_input(p.total, "uniform", seed + 1), np.full(5, 7.0)])
    for d in (0, 1):
        out = pre.copy()
        p(u, out, d)
        assert np.array_equal(out[p.total:], pre[p.total:])
        for v, N in enumerate(Ns):
            a, b = p.offsets[v], p.offsets[v + 1]
            w = pre[a:b].copy()
            orc.Oracle(N, maxs, 2).execute(np.ascontiguousarray(u[a:b]), w, d)
            assert relerr(out[a:b], w) <= TOL, (seed, v, N, maxs, d)


@pytest.mark.parametrize("seed", range(4))
def test_ragged_precompute_bitwise(lib, orc, seed):
    """Ragged lists made with precompute = 1 read the band weights from one
    table per leaf size (each table serving every vector with that leaf size,
    whatever its length): the bits of precompute = 0, and the oracle's results
    within the bar.  Lists mix lengths of one leaf size and direct vectors."""
    rng = np.random.default_rng(5000 + seed)
    count = int(rng.integers(20, 80))
    Ns = [int(n) for n in np.exp(rng.uniform(np.log(20), np.log(70000), count))]
    maxs = (64, 32, 50, 17)[seed]
    u = make_input(sum(Ns), "sign", seed + 9)
    outs = {}
    for pre in (0, 1):
        p = lib.RaggedPlan(Ns, maxs, precompute=pre)
        for d in (0, 1):
            out = np.zeros(p.total)
            p(u, out, d)
            outs[pre, d] = out
        p.close()
    offs = np.concatenate([[0], np.cumsum(Ns)])
    for d in (0, 1):
        assert np.array_equal(outs[1, d], outs[0, d]), (seed, d)
        for v in (0, count // 2, count - 1):
            a, b = offs[v], offs[v + 1]
            want = orc.Oracle(Ns[v], maxs, 2)(np.ascontiguousarray(u[a:b]), d)[:Ns[v]]
            assert relerr(outs[1, d][a:b], want) <= TOL, (seed, v, Ns[v], d)


def random_layout(seed):
    """The shape and layout draw of test_random_layouts_whole_buffer."""
    rng = np.random.default_rng(3000 + seed)
    form = ("modal", "nodal", "mixed")[seed % 3]
    N = int(np.exp(rng.uniform(np.log(2), np.log(70000))))
    maxs = int(rng.integers(8, 65))
    stride = int(rng.integers(1, 4))
    count = int(rng.integers(1, 13))
    dist = (N - 1) * stride + 1 + int(rng.integers(0, 40))
    return form, N, maxs, stride, count, dist


@pytest.mark.parametrize("seed", range(24))
def test_random_layouts_every_route_bitwise(lib, torch_cuda, seed):
    """The shapes and layouts of test_random_layouts_whole_buffer (checked
    there against the oracle) through every memory route: page-locked host
    buffers used in place, device arrays in place, and a plan with
    precompute = 1 (band weights from device memory; not for the mixed form,
    whose band is the same kernel) give the staged call's bits."""
    torch = torch_cuda
    form, N, maxs, stride, count, dist = random_layout(seed)
    lagrange = 1 if form == "nodal" else 0
    mixed = form == "mixed"
    size = count * dist + 7
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(size)
    pre = rng.uniform(-1, 1, size)  # incoming outputs: the transform adds to them
    p = lib.Plan(N, maxs, lagrange=lagrange, mixed=mixed)
    routes = {"pinned": lambda: (torch.from_numpy(x).pin_memory(),
                                 torch.from_numpy(pre.copy()).pin_memory()),
              "device": lambda: (torch.from_numpy(x).cuda(), torch.from_numpy(pre.copy()).cuda())}
    for d in (0, 1):
        want = pre.copy()
        p.execute_batched(x, want, d, count, dist, stride)
        for name, make in routes.items():
            for rep in range(2):  # capture, then replay
                xi, oi = make()
                p.execute_batched(xi, oi, d, count, dist, stride)
                torch.cuda.synchronize()
                assert np.array_equal(oi.cpu().numpy(), want), (name, rep, form, N, d)
        if not mixed and p.L >= 1:
            q = lib.Plan(N, maxs, lagrange=lagrange, precompute=1)
            got = pre.copy()
            q.execute_batched(x, got, d, count, dist, stride)
            assert np.array_equal(got, want), ("precompute", form, N, d)
            q.close()
    p.close()


@pytest.mark.parametrize("seed", range(8))
def test_random_2d_vs_lines(lib, orc, seed):
    """execute2D on seeded random array shapes (from direct-path sizes up),
    either axis, modal or nodal, precompute 0 or 1, against the oracle applied
    as the reference's execute2D applies execute() (leg2cheb.c:1267-1280):
    rows in place, columns one after another with stride N1.  For columns on
    the direct path (L = 0) that is not the line-by-line transform: each call
    zeroes [0, N0) and reads its L2C input contiguously from its column's
    start, reaching the neighbouring columns (sequential semantics, kept)."""
    rng = np.random.default_rng(5000 + seed)
    N0, N1 = (int(v) for v in np.exp(rng.uniform(np.log(2), np.log(700), 2)))
    axis = int(rng.integers(0, 2))
    maxs = int(rng.integers(8, 65))
    lagrange = int(rng.integers(0, 2))
    precompute = int(rng.integers(0, 2))
    x = np.ascontiguousarray(make_input(N0 * N1, "gauss", seed).reshape(N0, N1))
    p2 = lib.Plan2D(N0, N1, axis, maxs=maxs, lagrange=lagrange, precompute=precompute)
    n = (N0, N1)[axis]
    o = orc.Oracle(n, maxs, 2, lagrange=lagrange)
    why = (N0, N1, axis, maxs, lagrange, precompute)
    for d in (0, 1):
        out = np.zeros_like(x)
        p2(x, out, d)
        if axis == 0:
            xf, wf = x.ravel(), np.zeros(N0 * N1)
            for j in range(N1):  # views at column j's start: the reference's pointers
                o.execute(xf[j:], wf[j:], d, N1)
            want = wf.reshape(N0, N1)
        else:
            want = np.stack([o(np.ascontiguousarray(x[i]), d)[:N1] for i in range(N0)])
        assert relerr(out, want) <= TOL, why + (d,)
        if axis == 0 and o.L >= 1:  # FMM columns: the line-by-line transform
            lines = np.stack([o(np.ascontiguousarray(x[:, j]), d)[:N0] for j in range(N1)], axis=1)
            assert relerr(out, lines) <= TOL, why + (d,)


@pytest.mark.parametrize("N,maxs,lagrange", [(1 << 20, 64, 0), (1 << 16, 32, 0), (40000, 64, 0),
                                             (1 << 18, 16, 1), (20000, 24, 0), (30001, 64, 0),
                                             (9000, 21, 0), (3000, 10, 1)])
def test_single_vector_band_rows_vs_oracle(lib, orc, monkeypatch, N, maxs, lagrange):
    """The band's full blocks with register windows (rows of a block share
    their sources; leaf sizes not a multiple of 4 leave a partial row group:
    s = 59, 18, 6), forced on for every size (L2C_NEAR_ROWS=1; by default only
    vectors with many blocks take it); the same vector with the per-output
    kernel (L2C_NEAR_ROWS=0) and the oracle agree within the bar."""
    u = make_input(N, "sign", N + 3)
    o = orc.Oracle(N, maxs, 2, lagrange)
    outs = {}
    for env in ("1", "0"):
        with monkeypatch.context() as m:
            m.setenv("L2C_NEAR_ROWS", env)
            p = lib.Plan(N, maxs, lagrange=lagrange)
        for d in (0, 1):
            out = np.zeros(N)
            p.execute(u, out, d)
            outs[env, d] = out
        p.close()
    for d in (0, 1):
        want = o(u, d)[:N]
        assert relerr(outs["1", d], want) <= TOL, (N, d)
        assert relerr(outs["1", d], outs["0", d]) <= TOL, (N, d)
