"""Python front end of libleg2cheb.so (GB300 Legendre<->Chebyshev transform).

Mirrors the reference's ctypes wrapper (src/ctypes/l2ctypes.py): the same
``Leg2Cheb`` class with the same constructor arguments, defaults and call
signature, and the raw ``create_fmm`` / ``execute`` / ``create_direct`` /
``direct`` / ``Lambda`` bindings (l2ctypes.py:40-51).  On top of that:

* ``execute`` and ``execute_batched`` accept numpy arrays (host memory, copied
  to and from the GPU) or any object with ``data_ptr()`` (a CUDA torch tensor,
  used in place);
* failures raise ``L2CError`` with the library's message instead of crashing.

There is no CPU fallback: if the shared library is missing this module raises
on import of the library (``load()``).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")

L2C, C2L, BOTH = 0, 1, 2


class L2CError(RuntimeError):
    pass


_lib = None
_cuda = None


class _Opaque(ctypes.Structure):
    pass


def load():
    """Load libleg2cheb.so (and its libl2c_cuda.so); raise if not built."""
    global _lib, _cuda
    if _lib is not None:
        return _lib
    path = os.path.join(LIBDIR, "libleg2cheb.so")
    if not os.path.exists(path):
        raise L2CError(f"{path} is not built; run legendre-to-chebyshev_gb300/build.py")
    lib = ctypes.CDLL(path)
    cuda = ctypes.CDLL(os.path.join(LIBDIR, "libl2c_cuda.so"))
    sz, dp, vp = ctypes.c_size_t, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p
    lib.create_fmm.restype = vp
    lib.create_fmm.argtypes = [sz] * 7
    lib.create_fmm_ex.restype = vp
    lib.create_fmm_ex.argtypes = [sz] * 7 + [ctypes.c_uint]
    lib.free_fmm.argtypes = [vp]
    lib.execute.restype = sz
    lib.execute.argtypes = [vp, vp, vp, sz, sz]
    lib.execute_batched.restype = sz
    lib.execute_batched.argtypes = [vp, vp, vp, sz, sz, sz, sz]
    lib.create_direct.restype = vp
    lib.create_direct.argtypes = [sz, sz, sz]
    lib.free_direct.argtypes = [vp]
    lib.direct.restype = sz
    lib.direct.argtypes = [vp, vp, vp, sz, sz]
    lib.directM.restype = sz
    lib.directM.argtypes = [vp, vp, vp, sz]
    lib.directL.restype = sz
    lib.directL.argtypes = [vp, vp, vp, sz]
    lib.create_fmm_2d.restype = vp
    lib.create_fmm_2d.argtypes = [sz, sz, ctypes.c_int, sz, sz, sz, sz, sz, sz]
    lib.free_fmm_2d.argtypes = [vp]
    lib.execute2D.restype = sz
    lib.execute2D.argtypes = [vp, vp, vp, sz]
    for name in ("Lambda", "_Lambda0", "_LambdaE"):
        getattr(lib, name).restype = ctypes.c_double
        getattr(lib, name).argtypes = [ctypes.c_double]
    lib.LambdaI.restype = ctypes.c_double
    lib.LambdaI.argtypes = [sz]
    lib.Lambdavec.argtypes = [vp, vp, sz]
    lib.matvectri.argtypes = [vp, vp, vp, sz, ctypes.c_bool]
    lib.dct2.argtypes = [vp, vp]
    lib.l2c_last_error.restype = ctypes.c_char_p
    cuda.l2c_gpu_plan_create.restype = vp
    cuda.l2c_gpu_plan_create.argtypes = [sz, sz, sz, ctypes.c_uint]
    cuda.l2c_gpu_plan_destroy.argtypes = [vp]
    cuda.l2c_gpu_plan_info.restype = ctypes.c_int
    cuda.l2c_gpu_plan_info.argtypes = [vp, vp]
    cuda.l2c_gpu_execute.restype = sz
    cuda.l2c_gpu_execute.argtypes = [vp, vp, vp, sz, sz, sz, sz, ctypes.c_uint]
    cuda.l2c_gpu_synchronize.restype = ctypes.c_int
    cuda.l2c_gpu_synchronize.argtypes = [vp]
    cuda.l2c_gpu_plan_stream.restype = vp
    cuda.l2c_gpu_plan_stream.argtypes = [vp]
    cuda.l2c_gpu_flops.restype = sz
    cuda.l2c_gpu_flops.argtypes = [vp, sz]
    cuda.l2c_gpu_plan_copy.restype = sz
    cuda.l2c_gpu_plan_copy.argtypes = [vp, ctypes.c_int, vp, sz]
    cuda.l2c_geometry.restype = sz
    cuda.l2c_geometry.argtypes = [sz, sz, ctypes.POINTER(sz), ctypes.POINTER(sz)]
    lib.create_fmm_ragged.restype = vp
    lib.create_fmm_ragged.argtypes = [sz, vp, sz, sz, sz, sz, sz, sz]
    lib.execute_ragged.restype = sz
    lib.execute_ragged.argtypes = [vp, vp, vp, sz]
    lib.free_fmm_ragged.argtypes = [vp]
    cuda.l2c_gpu_ragged_execute.restype = sz
    cuda.l2c_gpu_ragged_execute.argtypes = [vp, vp, vp, sz, ctypes.c_uint]
    cuda.l2c_gpu_ragged_synchronize.restype = ctypes.c_int
    cuda.l2c_gpu_ragged_synchronize.argtypes = [vp]
    cuda.l2c_gpu_ragged_stream.restype = vp
    cuda.l2c_gpu_ragged_stream.argtypes = [vp]
    cuda.l2c_gpu_ragged_flops.restype = sz
    cuda.l2c_gpu_ragged_flops.argtypes = [vp, sz]
    cuda.l2c_gpu_ragged_launch_count.restype = sz
    cuda.l2c_gpu_ragged_launch_count.argtypes = [vp]
    cuda.l2c_gpu_last_error.restype = ctypes.c_char_p
    cuda.l2c_gpu_version.restype = ctypes.c_char_p
    cuda.l2c_gpu_ragged_autotune.restype = ctypes.c_double
    cuda.l2c_gpu_ragged_autotune.argtypes = [vp, sz]
    cuda.l2c_gpu_ragged_tuned_config.restype = ctypes.c_int
    cuda.l2c_gpu_ragged_tuned_config.argtypes = [vp, sz, ctypes.c_char_p, sz,
                                                 ctypes.POINTER(ctypes.c_double)]
    cuda.l2c_gpu_autotune.restype = ctypes.c_double
    cuda.l2c_gpu_autotune.argtypes = [vp, sz, sz, sz, sz]
    cuda.l2c_gpu_tuned_config.restype = ctypes.c_int
    cuda.l2c_gpu_tuned_config.argtypes = [vp, sz, sz, sz, sz, ctypes.c_char_p, sz,
                                          ctypes.POINTER(ctypes.c_double)]
    _lib, _cuda = lib, cuda
    return lib


def cuda_abi():
    load()
    return _cuda


def last_error():
    return load().l2c_last_error().decode()


def _ptr(a):
    """Address of a numpy array, of a tensor-like object with data_ptr(), or of
    any DLPack producer (``__dlpack__``: CuPy, JAX, ... device or host arrays,
    viewed without a copy)."""
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64:
            raise TypeError("arrays must be float64")
        return ctypes.c_void_p(a.ctypes.data)
    if hasattr(a, "__dlpack__"):
        import torch

        t = torch.utils.dlpack.from_dlpack(a)
        if t.dtype != torch.float64:
            raise TypeError("arrays must be float64")
        return ctypes.c_void_p(t.data_ptr())
    raise TypeError(f"unsupported array type {type(a)}")


def geometry(N, maxs):
    """(L, s, Nn) exactly as create_fmm computes them (leg2cheb.c:860-871)."""
    c = cuda_abi()
    s, nn = ctypes.c_size_t(), ctypes.c_size_t()
    L = c.l2c_geometry(N, maxs, ctypes.byref(s), ctypes.byref(nn))
    return int(L), int(s.value), int(nn.value)


class Plan:
    """An fmm_plan (create_fmm / free_fmm)."""

    def __init__(self, N, maxs=36, M=18, direction=BOTH, lagrange=0, precompute=0, verbose=0,
                 mixed=False):
        lib = load()
        self.N, self.maxs, self.direction = int(N), int(maxs), int(direction)
        self.mixed = bool(mixed)
        self._p = lib.create_fmm_ex(N, maxs, M, direction, lagrange, precompute, verbose,
                                    1 if mixed else 0)
        if not self._p:
            raise L2CError("create_fmm failed: " + last_error())
        gp = ctypes.cast(self._p, ctypes.POINTER(ctypes.c_void_p * 20)).contents[19]
        self._gpu = ctypes.c_void_p(gp)
        info = (ctypes.c_size_t * 8)()
        _cuda.l2c_gpu_plan_info(self._gpu, info)
        self.L, self.s, self.Nn, self.Nb = int(info[1]), int(info[2]), int(info[3]), int(info[4])

    @property
    def handle(self):
        return self._p

    @property
    def stream(self):
        return _cuda.l2c_gpu_plan_stream(self._gpu)

    def flops(self, direction):
        return int(_cuda.l2c_gpu_flops(self._gpu, direction))

    def execute(self, inp, out, direction, stride=1):
        f = _lib.execute(_ptr(inp), _ptr(out), self._p, direction, stride)
        if f == 0:
            raise L2CError("execute failed: " + last_error())
        return int(f)

    def execute_batched(self, inp, out, direction, count, dist, stride=1):
        f = _lib.execute_batched(_ptr(inp), _ptr(out), self._p, direction, count, dist, stride)
        if f == 0:
            raise L2CError("execute_batched failed: " + last_error())
        return int(f)

    def execute_async(self, inp, out, direction, count=1, dist=0, stride=1):
        """Queue on the plan's stream and return (device pointers only)."""
        f = _cuda.l2c_gpu_execute(self._gpu, _ptr(inp), _ptr(out), direction, count, dist,
                                  stride, 1)
        if f == 0:
            raise L2CError("l2c_gpu_execute failed: " + _cuda.l2c_gpu_last_error().decode())
        return int(f)

    def synchronize(self):
        if _cuda.l2c_gpu_synchronize(self._gpu) != 0:
            raise L2CError(_cuda.l2c_gpu_last_error().decode())

    def autotune(self, direction, count=1, dist=0, stride=1):
        """Tune the launch choices of one call shape (l2c_gpu_autotune); returns
        the tuned milliseconds per call.  Results are the same bits either way."""
        ms = _cuda.l2c_gpu_autotune(self._gpu, direction, count, dist, stride)
        if ms <= 0.0:
            raise L2CError("l2c_gpu_autotune failed: " + _cuda.l2c_gpu_last_error().decode())
        return float(ms)

    def tuned_config(self, direction, count=1, dist=0, stride=1):
        """(source, text, ms_tuned, ms_default) of a call shape's launch choices:
        source "tuned", "cache" or "default" (l2c_gpu_tuned_config)."""
        buf = ctypes.create_string_buffer(256)
        ms = (ctypes.c_double * 2)()
        r = _cuda.l2c_gpu_tuned_config(self._gpu, direction, count, dist, stride, buf, 256, ms)
        if r < 0:
            raise L2CError("l2c_gpu_tuned_config failed")
        return ({1: "tuned", 2: "cache"}.get(r, "default"), buf.value.decode(), ms[0], ms[1])

    def directM(self, inp, out, stride=1):
        f = _lib.directM(_ptr(inp), _ptr(out), self._p, stride)
        if f == 0:
            raise L2CError("directM failed: " + last_error())
        return int(f)

    def directL(self, inp, out, stride=1):
        f = _lib.directL(_ptr(inp), _ptr(out), self._p, stride)
        if f == 0:
            raise L2CError("directL failed: " + last_error())
        return int(f)

    def copy_table(self, which):
        """Plan data: 0 A[L2C], 1 A[C2L], 2 Lambda a, 3 an, 4 dn, 5 T,
        6 nodal transfer matrices B0 | B1 (nodal plans; empty otherwise)."""
        n = {0: 3 * self.Nb * 324, 1: 3 * self.Nb * 324, 2: self.N, 3: self.N,
             4: (self.N + 1) // 2, 5: 2 * self.s * 18, 6: 2 * 324}[which]
        buf = np.zeros(max(n, 1))
        got = _cuda.l2c_gpu_plan_copy(self._gpu, which, _ptr(buf), n)
        return buf[:got]

    def close(self):
        if getattr(self, "_p", None):
            _lib.free_fmm(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Leg2Cheb:
    """Legendre/Chebyshev transforms, as the reference's ctypes ``Leg2Cheb``
    (src/ctypes/l2ctypes.py:54-113): same arguments, defaults and behaviour.

    Parameters
    ----------
    input_array, output_array : numpy float64 arrays of length N
    maxs : int, max size of the smallest hierarchical block (default 36)
    M : int, rank of the hierarchical blocks (18)
    direction : 0 L2C, 1 C2L, 2 plan both
    """

    def __init__(self, input_array, output_array, maxs: int = 36, M: int = 18,
                 direction: int = 2, lagrange: int = 0, precompute: int = 0,
                 verbose: int = 1):
        self.N = input_array.shape[0]
        self.plan = Plan(self.N, maxs, M, direction, lagrange, precompute, verbose)
        self._input_array = input_array
        self._output_array = output_array

    def __call__(self, input_array=None, output_array=None, direction=0):
        assert direction in (0, 1)
        if input_array is not None:
            self._input_array[...] = input_array
        self._output_array[...] = 0
        self.plan.execute(self._input_array, self._output_array, direction, 1)
        if output_array is not None:
            output_array[...] = self._output_array
            return output_array
        return self._output_array


class RaggedPlan:
    """A ragged batch (create_fmm_ragged / execute_ragged / free_fmm_ragged):
    vectors of lengths Ns packed back to back, all transformed in one set of
    GPU launches."""

    def __init__(self, Ns, maxs=64, direction=BOTH, verbose=0, precompute=0):
        lib = load()
        self.Ns = np.asarray(Ns, dtype=np.uint64)
        self.offsets = np.concatenate([[0], np.cumsum(self.Ns)]).astype(np.int64)
        self.total = int(self.offsets[-1])
        arr = np.ascontiguousarray(self.Ns, dtype=np.uint64)
        self._p = lib.create_fmm_ragged(len(arr), arr.ctypes.data, maxs, 18, direction, 0,
                                        precompute, verbose)
        if not self._p:
            raise L2CError("create_fmm_ragged failed: " + last_error())
        self._gpu = ctypes.c_void_p(ctypes.cast(self._p, ctypes.POINTER(ctypes.c_void_p * 5))
                                    .contents[4])

    @property
    def stream(self):
        return _cuda.l2c_gpu_ragged_stream(self._gpu)

    def flops(self, direction):
        return int(_cuda.l2c_gpu_ragged_flops(self._gpu, direction))

    def launch_count(self):
        return int(_cuda.l2c_gpu_ragged_launch_count(self._gpu))

    def autotune(self, direction):
        """Tune this list's launch choices for one direction
        (l2c_gpu_ragged_autotune); returns the tuned ms per call."""
        ms = _cuda.l2c_gpu_ragged_autotune(self._gpu, direction)
        if ms <= 0.0:
            raise L2CError("l2c_gpu_ragged_autotune failed: " +
                           _cuda.l2c_gpu_last_error().decode())
        return float(ms)

    def tuned_config(self, direction):
        """(source, text, ms_tuned, ms_default): source "tuned" or "default"."""
        buf = ctypes.create_string_buffer(64)
        ms = (ctypes.c_double * 2)()
        r = _cuda.l2c_gpu_ragged_tuned_config(self._gpu, direction, buf, 64, ms)
        if r < 0:
            raise L2CError("l2c_gpu_ragged_tuned_config failed")
        return ("tuned" if r == 1 else "default", buf.value.decode(), ms[0], ms[1])

    def __call__(self, inp, out, direction):
        f = _lib.execute_ragged(_ptr(inp), _ptr(out), self._p, direction)
        if f == 0:
            raise L2CError("execute_ragged failed: " + last_error())
        return int(f)

    def execute_async(self, inp, out, direction):
        f = _cuda.l2c_gpu_ragged_execute(self._gpu, _ptr(inp), _ptr(out), direction, 1)
        if f == 0:
            raise L2CError(_cuda.l2c_gpu_last_error().decode())
        return int(f)

    def synchronize(self):
        if _cuda.l2c_gpu_ragged_synchronize(self._gpu) != 0:
            raise L2CError(_cuda.l2c_gpu_last_error().decode())

    def close(self):
        if getattr(self, "_p", None):
            _lib.free_fmm_ragged(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DirectPlan:
    """A direct_plan (create_direct / direct / free_direct): O(N^2) sums."""

    def __init__(self, N, direction=BOTH, precompute=0):
        lib = load()
        self.N = int(N)
        self._p = lib.create_direct(N, direction, precompute)
        if not self._p:
            raise L2CError("create_direct failed: " + last_error())

    def __call__(self, inp, out, direction, stride=1):
        f = _lib.direct(_ptr(inp), _ptr(out), self._p, direction, stride)
        if f == 0:
            raise L2CError("direct failed: " + last_error())
        return int(f)

    def close(self):
        if getattr(self, "_p", None):
            _lib.free_direct(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan2D:
    """An fmm_plan_2d (create_fmm_2d / execute2D / free_fmm_2d)."""

    def __init__(self, N0, N1, axis, maxs=36, M=18, direction=BOTH, verbose=0, lagrange=0,
                 precompute=0):
        lib = load()
        self._p = lib.create_fmm_2d(N0, N1, axis, maxs, M, direction, lagrange, precompute,
                                    verbose)
        if not self._p:
            raise L2CError("create_fmm_2d failed: " + last_error())

    def __call__(self, inp, out, direction):
        f = _lib.execute2D(_ptr(inp), _ptr(out), self._p, direction)
        if f == 0:
            raise L2CError("execute2D failed: " + last_error())
        return int(f)

    def close(self):
        if getattr(self, "_p", None):
            _lib.free_fmm_2d(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def Lambda(z):
    return load().Lambda(float(z))


def LambdaI(k):
    return load().LambdaI(int(k))
