"""Generate l2c_tables.h: the constant tables of the transform.

Run once when the tables change (needs mpmath and sympy, not needed at build
time; the generated header is committed).

* LAMBDA_INT[k] = Gamma(k+1/2)/Gamma(k+1), k < 256, correctly rounded (mpmath,
  60 digits).  Same values as the reference's integer table (lambda.c:101-191).
* LAMBDA_SERIES[k]: coefficients c_k of the large-z expansion
      Lambda(z) sqrt(z + 1/4) = sum_k c_k (z + 1/4)^(-2k),
  derived from the Stirling series of log Gamma with Bernoulli polynomials:
      log(Lambda(z) sqrt(t)) = sum_{n even} -2 B_{n+1}(1/4) / (n (n+1) t^n),  t = z + 1/4.
  The reference evaluates the same series (lambda.c:65-98).
* BINOM_LOWER / BINOM_UPPER: the 18x18 change-of-interval matrix
      C[i][j] = coefficient of T_j(x) in T_i((x - 1)/2)
  in compact lower (row-major, j <= i) and compact upper storage of its
  transpose (row i holds C[i..17][i]); exact dyadic rationals.  These are the
  reference's BMe / BMeT (leg2cheb.c:6-123).
"""
import os
from fractions import Fraction

import mpmath
import sympy as sp

M = 18
HERE = os.path.dirname(os.path.abspath(__file__))


def lambda_int():
    mpmath.mp.dps = 60
    return [float(mpmath.gamma(k + mpmath.mpf(1) / 2) / mpmath.gamma(k + 1)) for k in range(256)]


def lambda_series(nterms=7):
    w = sp.symbols("w")
    quarter = sp.Rational(1, 4)
    log_series = 0
    for n in range(2, 2 * nterms + 1, 2):
        log_series += -2 * sp.bernoulli(n + 1, quarter) / (n * (n + 1)) * w ** (n // 2)
    ser = sp.series(sp.exp(log_series), w, 0, nterms).removeO()
    return [sp.Rational(ser.coeff(w, k)) for k in range(nterms)]


def cheb_shift_matrix():
    # Chebyshev-basis coefficient vectors; y = (x - 1)/2.
    def times_x(c):
        out = [Fraction(0)] * (len(c) + 1)
        for j, v in enumerate(c):
            if j == 0:
                out[1] += v
            else:
                out[j + 1] += v / 2
                out[j - 1] += v / 2
        return out

    def add(a, b, sa=1, sb=1):
        n = max(len(a), len(b))
        a = a + [Fraction(0)] * (n - len(a))
        b = b + [Fraction(0)] * (n - len(b))
        return [sa * x + sb * y for x, y in zip(a, b)]

    polys = [[Fraction(1)], [Fraction(-1, 2), Fraction(1, 2)]]
    while len(polys) < M:
        p1, p0 = polys[-1], polys[-2]
        two_y_p1 = add(times_x(p1), p1, 1, -1)  # 2y T_i = (x - 1) T_i
        polys.append(add(two_y_p1, p0, 1, -1))
    C = [[Fraction(0)] * M for _ in range(M)]
    for i, p in enumerate(polys):
        for j, v in enumerate(p[:M]):
            C[i][j] = v
    return C


def fmt(x):
    return float(x).hex()


def main():
    li = lambda_int()
    ser = lambda_series()
    C = cheb_shift_matrix()
    lower = [C[i][j] for i in range(M) for j in range(i + 1)]
    upper = [C[j][i] for i in range(M) for j in range(i, M)]
    for v in lower + upper:
        assert Fraction(float(v)) == v, "binomial entry not exact in double"
    lines = [
        "/* Generated by gen_tables.py -- do not edit. */",
        "#ifndef L2C_TABLES_H",
        "#define L2C_TABLES_H",
        "",
        "/* Gamma(k+1/2)/Gamma(k+1), k < 256, correctly rounded. */",
        "#define L2C_LAMBDA_INT_INIT { \\",
    ]
    for k in range(0, 256, 4):
        lines.append("  " + ", ".join(fmt(v) for v in li[k:k + 4]) + ", \\")
    lines.append("}")
    lines.append("")
    lines.append("/* Lambda(z) sqrt(z+1/4) = sum_k c_k (z+1/4)^(-2k); c_k exact (dyadic). */")
    for k, c in enumerate(ser):
        assert Fraction(float(c)) == Fraction(c.p, c.q)
        lines.append(f"#define L2C_LAMBDA_C{k} {fmt(c)} /* {c} */")
    lines.append("")
    lines.append("/* C[i][j] = coefficient of T_j(x) in T_i((x-1)/2): compact lower, row-major. */")
    lines.append("#define L2C_BINOM_LOWER_INIT { \\")
    for k in range(0, len(lower), 4):
        lines.append("  " + ", ".join(fmt(v) for v in lower[k:k + 4]) + ", \\")
    lines.append("}")
    lines.append("/* Transpose of C in compact upper storage: row i holds C[i..17][i]. */")
    lines.append("#define L2C_BINOM_UPPER_INIT { \\")
    for k in range(0, len(upper), 4):
        lines.append("  " + ", ".join(fmt(v) for v in upper[k:k + 4]) + ", \\")
    lines.append("}")
    lines.append("")
    lines.append("#endif")
    with open(os.path.join(HERE, "l2c_tables.h"), "w") as f:
        f.write("\n".join(lines) + "\n")
    print("series:", ser)


if __name__ == "__main__":
    main()
