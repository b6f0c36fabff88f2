"""l2c_gpu_execute_noalloc: one transform with no device allocation.

Callers that cannot allocate device memory while they transform (an application
that owns the whole device through its own pool, a time-stepping solver that
must not risk allocation latency or failure mid-step) get an entry point whose
working buffers live in a fixed array inside the library.  Here it is called
through the C ABI and compared with the ordinary entry point, l2c_gpu_execute,
and with the oracle port, on two calls in a row (the second call reuses the
array the first one left behind); a fresh plan's first call must leave the
device's free memory unchanged; two threads calling at once must both get
right answers (the calls are serialised per device).  Kept in its own file,
collected last."""
import ctypes
import threading

import numpy as np
import pytest

from tests.conftest import relerr
from tests.golden.cases import make_input

pytestmark = pytest.mark.gpu

TOL = 1e-14


def _abi(lib):
    c = lib.cuda_abi()
    c.l2c_gpu_execute_noalloc.restype = ctypes.c_size_t
    c.l2c_gpu_execute_noalloc.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_size_t] * 2
    return c


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("N,maxs,stride,lagrange", [(4096, 64, 1, 0), (65536, 32, 1, 0),
                                                    (5001, 64, 3, 0), (16384, 32, 1, 1)])
def test_noalloc_matches_execute_two_calls(lib, N, maxs, stride, lagrange):
    import torch

    c = _abi(lib)
    p = lib.Plan(N, maxs, lagrange=lagrange)
    for d in (0, 1):
        inputs = [make_input(N * stride, "uniform", 10 + d), make_input(N * stride, "sign", 20 + d)]
        for u in inputs:  # two calls in a row
            du = torch.from_numpy(u).cuda()
            want = torch.zeros(N * stride, dtype=torch.float64, device="cuda")
            got = torch.zeros_like(want)
            assert c.l2c_gpu_execute(p._gpu, ctypes.c_void_p(du.data_ptr()),
                                     ctypes.c_void_p(want.data_ptr()), d, 1, 0, stride, 0)
            f = c.l2c_gpu_execute_noalloc(p._gpu, ctypes.c_void_p(du.data_ptr()),
                                          ctypes.c_void_p(got.data_ptr()), d, stride)
            assert f == p.flops(d), c.l2c_gpu_last_error().decode()
            assert relerr(got.cpu().numpy(), want.cpu().numpy()) <= TOL


def test_noalloc_rejects_plans_beyond_the_fixed_array(lib):
    import torch

    c = _abi(lib)
    N = 1 << 20
    p = lib.Plan(N, 64)
    du = torch.zeros(N, dtype=torch.float64, device="cuda")
    out = torch.zeros_like(du)
    assert c.l2c_gpu_execute_noalloc(p._gpu, ctypes.c_void_p(du.data_ptr()),
                                     ctypes.c_void_p(out.data_ptr()), 0, 1) == 0
    assert "too large" in c.l2c_gpu_last_error().decode()


def test_noalloc_rejects_host_pointers(lib):
    c = _abi(lib)
    p = lib.Plan(4096, 64)
    u, out = np.ones(4096), np.zeros(4096)
    assert c.l2c_gpu_execute_noalloc(p._gpu, ctypes.c_void_p(u.ctypes.data),
                                     ctypes.c_void_p(out.ctypes.data), 0, 1) == 0
    assert "device pointers" in c.l2c_gpu_last_error().decode()


def test_fresh_plan_first_call_allocates_nothing(lib, orc):
    """A fresh plan (no call made on it yet, so none of its grown-on-demand
    buffers exists) whose first call is the no-allocation entry point: the
    device's free memory is the same before and after the call, and the result
    matches the oracle and a later l2c_gpu_execute.  The scratch the ordinary
    path would grow for this plan is about 2.8 MB, above the driver's
    allocation granularity, so a fallback to it would show."""
    import torch

    c = _abi(lib)
    N, maxs = 100000, 64
    # load the kernels this entry point launches, on a throwaway plan first
    warm = lib.Plan(N, maxs)
    wu = torch.ones(N, dtype=torch.float64, device="cuda")
    wo = torch.zeros_like(wu)
    assert c.l2c_gpu_execute_noalloc(warm._gpu, _vp(wu), _vp(wo), 0, 1)
    warm.close()
    u = make_input(N, "uniform", 99)
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        p = lib.Plan(N, maxs)
        du = torch.from_numpy(u).cuda()
        got = torch.zeros_like(du)
        want = torch.zeros_like(du)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        f = c.l2c_gpu_execute_noalloc(p._gpu, _vp(du), _vp(got), d, 1)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert f == p.flops(d), c.l2c_gpu_last_error().decode()
        assert free1 == free0, (d, free0 - free1)
        assert relerr(got.cpu().numpy(), o(u, d)[:N]) <= TOL
        assert c.l2c_gpu_execute(p._gpu, _vp(du), _vp(want), d, 1, 0, 1, 0)
        p.synchronize()
        assert relerr(got.cpu().numpy(), want.cpu().numpy()) <= TOL
        p.close()


def test_mixed_plan_runs_fp64_far_field(lib, orc):
    """On a mixed-form plan the entry point runs the FP64 far field: the
    results agree with the oracle and with l2c_gpu_execute's mixed-form results
    within the 1e-14 bar."""
    import torch

    c = _abi(lib)
    N, maxs = 16384, 16
    p = lib.Plan(N, maxs, mixed=True)
    o = orc.Oracle(N, maxs, 2)
    for d in (0, 1):
        for seed in (5, 6):  # two calls in a row
            u = make_input(N, "gauss", seed)
            du = torch.from_numpy(u).cuda()
            got = torch.zeros_like(du)
            want = torch.zeros_like(du)
            assert c.l2c_gpu_execute_noalloc(p._gpu, _vp(du), _vp(got), d, 1) == p.flops(d)
            assert c.l2c_gpu_execute(p._gpu, _vp(du), _vp(want), d, 1, 0, 1, 0)
            p.synchronize()
            assert relerr(got.cpu().numpy(), o(u, d)[:N]) <= TOL
            assert relerr(got.cpu().numpy(), want.cpu().numpy()) <= TOL


def test_two_threads_at_once(lib, orc):
    """Two host threads, each with its own plan and inputs, calling the entry
    point several times at once (ctypes releases the GIL, so the calls overlap
    on the host; the library serialises them on the device because they share
    the fixed array).  Every result matches the oracle."""
    import torch

    c = _abi(lib)
    cases = [(4096, 64, 31), (12000, 32, 32)]
    plans = [lib.Plan(N, maxs) for N, maxs, _ in cases]
    wants = []
    inputs = []
    for N, maxs, seed in cases:
        u = make_input(N, "uniform", seed)
        o = orc.Oracle(N, maxs, 2)
        inputs.append(u)
        wants.append([o(u, d)[:N] for d in (0, 1)])
    errors = []

    def worker(i):
        try:
            N = cases[i][0]
            du = torch.from_numpy(inputs[i]).cuda()
            outs = [torch.zeros_like(du) for _ in range(2)]
            torch.cuda.synchronize()
            for _ in range(6):
                for d in (0, 1):
                    outs[d].zero_()
                    torch.cuda.synchronize()
                    if not c.l2c_gpu_execute_noalloc(plans[i]._gpu, _vp(du), _vp(outs[d]), d, 1):
                        errors.append((i, d, c.l2c_gpu_last_error().decode()))
                        return
                    e = relerr(outs[d].cpu().numpy(), wants[i][d])
                    if not e <= TOL:
                        errors.append((i, d, N, e))
        except Exception as exc:  # reported by the main thread
            errors.append((i, repr(exc)))

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
