"""l2c_gpu_execute_noalloc: one transform with no device allocation.

Callers that cannot allocate device memory while they transform (an application
that owns the whole device through its own pool, a time-stepping solver that
must not risk allocation latency or failure mid-step) get an entry point whose
working buffers live in a fixed array inside the library.  Here it is called
through the C ABI and compared with the ordinary entry point, l2c_gpu_execute,
on two calls in a row (the second call reuses the array the first one left
behind).  Kept in its own file, collected last."""
import ctypes

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
