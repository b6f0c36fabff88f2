"""TEST INFRASTRUCTURE -- extended-precision direct O(N^2) transforms.

Restates the reference's multiprecision checkers (src/multiprec/C++/L2Cprec.cpp:19-69
and src/multiprec/python/L2Cprecision.py:10-33) in numpy ``longdouble``
(80-bit on x86-64, IEEE quad on aarch64), for parity checks at N <= ~16384.

    L2C:  b_i = (2/pi) sum_{n even} Lambda(n/2) Lambda(n/2 + i) u_{i+n},   b_0 /= 2
    C2L:  b_i = (i + 1/2) [ sqrt(pi) an_i v_i - sum_{k>=1} dn_k an_{i+k} v_{i+2k} ]
          v_0 = u_0, v_j = j u_j,  an_0 = 2/sqrt(pi),  an_i = 1/(Lambda(i)(2i^2+i)),
          dn_k = Lambda(k-1)/(2k)                       (leg2cheb.c:152-234, 781-795)

Lambda(k) = Gamma(k+1/2)/Gamma(k+1) comes from the exact ratio
Lambda(k+1) = Lambda(k) (k+1/2)/(k+1), started at sqrt(pi), in long double.
"""
import numpy as np

LD = np.longdouble
_PI = LD("3.14159265358979323846264338327950288419716939937510")
_SQRT_PI = LD("1.77245385090551602729816748334114518279754945612239")


def lambda_table(n):
    """Lambda(k) for k < n in long double."""
    n = max(int(n), 1)
    k = np.arange(n - 1, dtype=LD)
    ratios = (k + LD(0.5)) / (k + LD(1))
    out = np.empty(n, dtype=LD)
    out[0] = _SQRT_PI
    out[1:] = _SQRT_PI * np.cumprod(ratios)
    return out


def l2c_direct(u):
    """Extended-precision L2C of one vector; returns long double array."""
    u = np.asarray(u, dtype=LD)
    N = u.shape[0]
    a = lambda_table(N)
    b = np.zeros(N, dtype=LD)
    for n in range(0, N, 2):
        k = n // 2
        b[: N - n] += a[k] * a[k : k + N - n] * u[n:]
    b *= LD(2) / _PI
    b[0] /= 2
    return b


def c2l_direct(u):
    """Extended-precision C2L of one vector; returns long double array."""
    u = np.asarray(u, dtype=LD)
    N = u.shape[0]
    a = lambda_table(N + 1)
    i = np.arange(N, dtype=LD)
    v = u * i
    v[0] = u[0]
    an = np.empty(N, dtype=LD)
    an[0] = LD(2) / _SQRT_PI
    an[1:] = LD(1) / (a[1:N] * (2 * i[1:] * i[1:] + i[1:]))
    b = _SQRT_PI * an * v
    for k in range(1, (N + 1) // 2):
        dk = a[k - 1] / (2 * k)
        b[: N - 2 * k] -= dk * an[k : N - k] * v[2 * k :]
    b *= i + LD(0.5)
    return b


def rel_maxnorm(x, ref):
    """max|x - ref| / max|ref| evaluated in long double."""
    x = np.asarray(x, dtype=LD)
    ref = np.asarray(ref, dtype=LD)
    den = np.max(np.abs(ref))
    return float(np.max(np.abs(x - ref)) / (den if den != 0 else LD(1)))
