"""GPU parity at the exact benchmark workloads.

Every workload bench.py times is run here on its own seeded inputs
(bench.Workload, seed 1 as on rank 0), at its own shapes and leaf sizes, and
EVERY output vector is compared with the oracle port (oracle/l2c_oracle.c, a
restatement of leg2cheb.c:1299-1500 pinned against the unmodified reference's
golden vectors) per direction, at 1e-14 relative max-norm
(max|y - y_ref| / max|y_ref|, per vector):

  * N = 512 round trip, maxs 64 and 32 (like `l2c -N512 -d2`)
  * single vectors N = 2^10 ... 2^24, c_n = s_n/(n+1), maxs 64
  * 4096 lines of N = 1024 (a 64x64x1024 array), L2C then C2L of the result
  * the ragged list: 2000 vectors, N log-uniform in [64, 65536]
  * mixed form (maxs 16) against plain FP64 (maxs 16, 32, 64) on the same
    inputs: a single N = 2^22 and 256 vectors of N = 16384, iid N(0, 1)

Where the reference itself was built on this machine (oracle/_ref, from its
unmodified sources), single vectors up to N = 2^24 are also compared with the
reference's own execute() directly.
"""
import ctypes
import os

import numpy as np
import pytest

import bench
from tests.conftest import REPO, relerr
from tests.golden.cases import make_input

pytestmark = pytest.mark.gpu

TOL = 1e-14


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    return torch


def per_vector_relerr(got, want):
    """Relative max-norm error of each row."""
    got = np.atleast_2d(got)
    want = np.atleast_2d(want)
    den = np.max(np.abs(want), axis=1)
    den[den == 0] = 1.0
    return np.max(np.abs(got - want), axis=1) / den


@pytest.mark.parametrize("maxs", [64, 32])
def test_n512_round_trip(lib, orc, maxs):
    N = 512
    u = np.random.default_rng(1).uniform(-1.0, 1.0, N)
    p = lib.Plan(N, maxs)
    o = orc.Oracle(N, maxs, 2)
    b = np.zeros(N)
    p.execute(u, b, 0)
    assert relerr(b, o(u, 0)[:N]) <= TOL
    c = np.zeros(N)
    p.execute(b, c, 1)
    assert relerr(c, o(b, 1)[:N]) <= TOL
    # src/bin/l2c.c:58-60 asks 1e-10 of the round trip; it is far below that
    assert relerr(c, u) <= 1e-12


@pytest.mark.parametrize("k", list(range(10, 25)))
def test_single_vector_sweep(lib, orc, torch_cuda, k):
    torch = torch_cuda
    N = 1 << k
    wl = bench.Workload("single", N, 64, 1)
    du = torch.from_numpy(np.ascontiguousarray(wl.u[0])).cuda()
    p = lib.Plan(N, 64)
    o = orc.Oracle(N, 64, 2)
    for d in (0, 1):
        out = torch.zeros_like(du)
        p.execute(du, out, d)
        assert relerr(out.cpu().numpy(), o(wl.u[0], d)[:N]) <= TOL, (N, d)
    p.close()
    o.close()


def test_lines_of_3d_array_every_line(lib, orc, torch_cuda):
    torch = torch_cuda
    wl = bench.Workload("batch", 1024, 64, 1)
    count, N = wl.count, wl.N
    x = np.ascontiguousarray(wl.u)
    p = lib.Plan(N, 64)
    o = orc.Oracle(N, 64, 2)
    dx = torch.from_numpy(x).cuda()
    dy, dz = torch.zeros_like(dx), torch.zeros_like(dx)
    p.execute_batched(dx, dy, 0, count, N, 1)
    y = dy.cpu().numpy()
    want = np.zeros_like(x)
    o.execute_batch(x, want, 0, count, N)
    assert per_vector_relerr(y, want).max() <= TOL
    p.execute_batched(dy, dz, 1, count, N, 1)
    z = dz.cpu().numpy()
    want = np.zeros_like(x)
    o.execute_batch(y, want, 1, count, N)
    assert per_vector_relerr(z, want).max() <= TOL
    assert relerr(z, x) <= 1e-13


def test_ragged_list_every_vector(lib, orc):
    wl = bench.Workload("ragged", 1024, 64, 1)
    u = np.ascontiguousarray(wl.u[0])
    p = lib.RaggedPlan(wl.Ns, 64)
    ro = orc.RaggedOracle(wl.Ns, 64, 2)
    off = p.offsets
    for d in (0, 1):
        out = np.zeros_like(u)
        p(u, out, d)
        want = np.zeros_like(u)
        ro.execute(u, want, d)
        for v in range(len(wl.Ns)):
            a, b = int(off[v]), int(off[v + 1])
            e = relerr(out[a:b], want[a:b])
            assert e <= TOL, (d, v, int(wl.Ns[v]), e)
    p.close()


@pytest.mark.parametrize("maxs,mixed", [(16, True), (16, False), (32, False), (64, False)])
@pytest.mark.parametrize("workload,N", [("mixed_batch", 16384), ("mixed_single", 1 << 22)])
def test_mixed_and_plain_same_inputs(lib, orc, torch_cuda, workload, N, maxs, mixed):
    torch = torch_cuda
    wl = bench.Workload(workload, N, maxs, 1)
    count = wl.count
    x = np.ascontiguousarray(wl.u)
    p = lib.Plan(N, maxs, mixed=mixed)
    o = orc.Oracle(N, maxs, 2)
    dx = torch.from_numpy(x).cuda()
    for d in (0, 1):
        dout = torch.zeros_like(dx)
        p.execute_batched(dx, dout, d, count, N, 1)
        want = np.zeros_like(x)
        if count == 1:
            o.execute(x[0], want[0], d)
        else:
            o.execute_batch(x, want, d, count, N)
        errs = per_vector_relerr(dout.cpu().numpy(), want)
        assert errs.max() <= TOL, (workload, maxs, mixed, d, int(errs.argmax()), errs.max())
    p.close()
    o.close()


REF_DIR = os.path.join(REPO, "oracle", "_ref")


@pytest.fixture(scope="module")
def reference():
    """The reference's own execute(), built from its unmodified sources into
    oracle/_ref (oracle/Makefile; skipped where it was not built)."""
    path = os.path.join(REF_DIR, "libleg2cheb_ref.so")
    if not (os.path.exists(path) and os.path.exists(os.path.join(REF_DIR, "libref_batch.so"))):
        pytest.skip("the reference was not built on this machine")
    sz, vp = ctypes.c_size_t, ctypes.c_void_p
    ref = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    ref.create_fmm.restype = vp
    ref.create_fmm.argtypes = [sz] * 7
    ref.execute.restype = sz
    ref.execute.argtypes = [vp, vp, vp, sz, sz]
    ref.free_fmm.argtypes = [vp]
    batch = ctypes.CDLL(os.path.join(REF_DIR, "libref_batch.so"))
    batch.ref_set_threads.argtypes = [ctypes.c_int, ctypes.c_int]
    batch.ref_set_threads(os.cpu_count() or 1, 1)
    return ref


@pytest.mark.parametrize("N,maxs,dist,lagrange", [
    (512, 32, "uniform", 0), (1024, 64, "gauss2", 0), (16384, 16, "gauss", 0),
    (1 << 20, 64, "sign", 0), (1 << 20, 64, "sign", 1), (1 << 22, 16, "gauss", 0),
    (1 << 24, 64, "sign", 0)])
def test_matches_reference_execute(lib, reference, torch_cuda, N, maxs, dist, lagrange):
    """Against the reference's own execute() on the same inputs, per direction
    (its flop count too)."""
    torch = torch_cuda
    u = make_input(N, dist, N + maxs)
    p = lib.Plan(N, maxs, lagrange=lagrange)
    rp = reference.create_fmm(N, maxs, 18, 2, lagrange, 0, 0)
    assert rp
    du = torch.from_numpy(u).cuda()
    for d in (0, 1):
        want = np.zeros(N + 8)  # the reference's odd-N scatter writes past N
        flops = reference.execute(u.ctypes.data, want.ctypes.data, rp, d, 1)
        out = torch.zeros_like(du)
        assert p.execute(du, out, d) == flops
        assert relerr(out.cpu().numpy(), want[:N]) <= TOL, (N, maxs, d)
    reference.free_fmm(rp)
    p.close()
