"""TEST INFRASTRUCTURE -- ctypes loader for the oracle port (l2c_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
``Oracle(N, maxs, direction)`` mirrors create_fmm/execute/free_fmm of the
reference (see l2c_oracle.h for the function-by-function citations).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborc.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    src = os.path.join(HERE, "l2c_oracle.c")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        build()
    lib = ctypes.CDLL(LIB)
    sz, vp = ctypes.c_size_t, ctypes.c_void_p
    lib.orc_create.restype = vp
    lib.orc_create.argtypes = [sz, sz, sz]
    lib.orc_create_ex.restype = vp
    lib.orc_create_ex.argtypes = [sz, sz, sz, sz]
    lib.orc_free.argtypes = [vp]
    lib.orc_execute.restype = sz
    lib.orc_execute.argtypes = [vp, vp, vp, sz, sz]
    lib.orc_plan_info.argtypes = [vp, vp]
    lib.orc_execute_batch.restype = sz
    lib.orc_execute_batch.argtypes = [vp, vp, vp, sz, sz, sz, sz]
    lib.orc_execute_ragged.restype = sz
    lib.orc_execute_ragged.argtypes = [vp, vp, vp, vp, sz, sz]
    for name in ("orc_directM", "orc_directL"):
        getattr(lib, name).restype = sz
        getattr(lib, name).argtypes = [vp, vp, vp, sz]
    for name in ("orc_plan_A",):
        getattr(lib, name).restype = ctypes.POINTER(ctypes.c_double)
        getattr(lib, name).argtypes = [vp, sz]
    for name in ("orc_plan_T", "orc_plan_lambda", "orc_plan_B", "orc_plan_BT"):
        getattr(lib, name).restype = ctypes.POINTER(ctypes.c_double)
        getattr(lib, name).argtypes = [vp]
    lib.orc_Lambda.restype = ctypes.c_double
    lib.orc_Lambda.argtypes = [ctypes.c_double]
    lib.orc_LambdaI.restype = ctypes.c_double
    lib.orc_LambdaI.argtypes = [sz]
    lib.orc_set_threads.argtypes = [ctypes.c_int]
    lib.orc_uses_blas.restype = ctypes.c_int
    _lib = lib
    return lib


class Oracle:
    def __init__(self, N, maxs=64, direction=2, lagrange=0):
        lib = load()
        self.N = int(N)
        self.lagrange = int(lagrange)
        self._p = lib.orc_create_ex(N, maxs, direction, self.lagrange)
        info = (ctypes.c_size_t * 6)()
        lib.orc_plan_info(self._p, info)
        self.L, self.s, self.Nn, self.Nb = int(info[1]), int(info[2]), int(info[3]), int(info[4])

    def execute(self, u, out, direction, stride=1):
        """out is updated in place (needs room for (N-1)*stride + 1 doubles)."""
        assert u.dtype == np.float64 and out.dtype == np.float64
        return int(load().orc_execute(u.ctypes.data, out.ctypes.data, self._p, direction, stride))

    def __call__(self, u, direction, stride=1):
        out = np.zeros(max(len(u), (self.N - 1) * stride + 1))
        self.execute(np.ascontiguousarray(u, dtype=np.float64), out, direction, stride)
        return out

    def execute_batch(self, u, out, direction, count, dist, stride=1):
        assert u.dtype == np.float64 and out.dtype == np.float64
        return int(load().orc_execute_batch(u.ctypes.data, out.ctypes.data, self._p, direction,
                                            count, dist, stride))

    def directM(self, u, out, stride=1):
        return int(load().orc_directM(u.ctypes.data, out.ctypes.data, self._p, stride))

    def directL(self, v, out, stride=1):
        return int(load().orc_directL(v.ctypes.data, out.ctypes.data, self._p, stride))

    def A(self, direction):
        p = load().orc_plan_A(self._p, direction)
        if not p:
            return None
        return np.ctypeslib.as_array(p, (3 * self.Nb * 324,)).copy()

    def lambda_table(self):
        return np.ctypeslib.as_array(load().orc_plan_lambda(self._p), (self.N,)).copy()

    def T(self):
        return np.ctypeslib.as_array(load().orc_plan_T(self._p), (2 * self.s * 18,)).copy()

    def B(self):
        """Transfer matrices: compact binomial (171, modal) or B0 | B1 (648, nodal)."""
        n = 2 * 324 if self.lagrange else 171
        return np.ctypeslib.as_array(load().orc_plan_B(self._p), (n,)).copy()

    def close(self):
        if getattr(self, "_p", None):
            load().orc_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_threads(n):
    load().orc_set_threads(int(n))


def uses_blas():
    return bool(load().orc_uses_blas())


class RaggedOracle:
    """Per-vector oracle plans for a ragged list (plans shared between equal N)."""

    def __init__(self, Ns, maxs=64, direction=2):
        self.Ns = [int(n) for n in Ns]
        cache = {}
        self.plans = []
        for n in self.Ns:
            if n not in cache:
                cache[n] = Oracle(n, maxs, direction)
            self.plans.append(cache[n])
        self._keep = cache
        self.offsets = np.concatenate([[0], np.cumsum(self.Ns)]).astype(np.uint64)
        self._pp = (ctypes.c_void_p * len(self.plans))(*[p._p for p in self.plans])

    def execute(self, u, out, direction):
        return int(load().orc_execute_ragged(u.ctypes.data, out.ctypes.data, self._pp,
                                             self.offsets.ctypes.data, len(self.Ns), direction))
