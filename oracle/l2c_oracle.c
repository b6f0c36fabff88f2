/* TEST INFRASTRUCTURE -- not part of the shipped library.
 *
 * CPU restatement of the reference fast multipole Legendre<->Chebyshev
 * transform (spectralDNS/Legendre-to-Chebyshev).  See l2c_oracle.h.  Built with
 * -ffp-contract=off so its rounding follows the reference's plain C on x86-64.
 * OpenMP parallelises the same loops the reference parallelises, so the port
 * also serves as the CPU baseline on machines where the reference itself
 * cannot be built. */
#include "l2c_oracle.h"

#ifdef ORC_CBLAS
/* The reference calls CBLAS dgemm for steps 1 and 5 (leg2cheb.c:1381, 1467);
 * with ORC_CBLAS the port does the same through the OpenBLAS that scipy bundles
 * (its CBLAS symbols carry a "scipy_" prefix), single-threaded inside OpenMP row
 * blocks (OpenBLAS's own thread pool and OpenMP's oversubscribe the cores).  Step 3's 18x18 products stay in
 * the port's OpenMP loop: the reference's dgemv calls inside an OpenMP loop
 * (leg2cheb.c:1419-1435) serialise in OpenBLAS's thread server, an 8x slowdown
 * on 8 threads, which would not be a fair baseline. */
enum { OrcRowMajor = 101 };
enum { OrcNoTrans = 111, OrcTrans = 112 };
void scipy_cblas_dgemm(int, int, int, int, int, int, double, const double *, int, const double *,
                       int, double, double *, int);
void scipy_openblas_set_num_threads(int);
#endif

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_M 18
#define ORC_MM (ORC_M * ORC_M)
#define ORC_NTRI ((ORC_MM + ORC_M) / 2)

struct orc_plan {
  size_t N, L, s, Nn, Nb, dirs; /* dirs: ORC_L2C, ORC_C2L or ORC_BOTH */
  size_t lagrange;              /* 0 modal, 1 nodal                     */
  double *a;                    /* Lambda(i), i < N                     */
  double *an, *dn;              /* C2L tables (NULL for an L2C plan)    */
  double *A[2];                 /* far-field blocks per direction       */
  double *T;                    /* leaf matrices, even rows then odd    */
  double B[ORC_NTRI], BT[ORC_NTRI];
  double LB[2 * ORC_MM];        /* nodal: child interpolation B0 | B1   */
};

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
#ifdef ORC_CBLAS
  (void)n;
  scipy_openblas_set_num_threads(1); /* threads come from OpenMP row blocks */
#endif
}

int orc_uses_blas(void) {
#ifdef ORC_CBLAS
  return 1;
#else
  return 0;
#endif
}

/* ---------------------------------------------------------------------------
 * Lambda(z) = Gamma(z+1/2)/Gamma(z+1).
 * lambda.c:65-98: for z < 10 recurse upward with Lambda(z) = Lambda(z+1)(z+1)/(z+1/2);
 * otherwise the asymptotic series in w = (z+1/4)^-2,
 *   Lambda(z) sqrt(z+1/4) = 1 - w/64 + 21w^2/8192 - 671w^3/524288
 *                          + 180323w^4/134217728 - 20898423w^5/8589934592
 *                          + 7426362705w^6/1099511627776,
 * truncated after fewer terms for larger z (cut points 2014, 141, 40, 20, 14).
 * ------------------------------------------------------------------------- */
double orc_Lambda(double z) {
  if (z < 10) return orc_Lambda(z + 1) * (z + 1) / (z + 0.5);
  const double zp = z + 0.25;
  const double sc = 1 / sqrt(zp);
  const double w = 1 / (zp * zp);
  static const double c1 = 1.0 / 64, c2 = 21.0 / 8192, c3 = 671.0 / 524288,
                      c4 = 180323.0 / 134217728, c5 = 20898423.0 / 8589934592.0,
                      c6 = 7426362705.0 / 1099511627776.0;
  double y = 1 - c1 * w;
  if (z > 2014) return y * sc;
  double wk = w * w;
  y += c2 * wk;
  if (z > 141) return y * sc;
  wk *= w;
  y -= c3 * wk;
  if (z > 40) return y * sc;
  wk *= w;
  y += c4 * wk;
  if (z > 20) return y * sc;
  wk *= w;
  y -= c5 * wk;
  if (z > 14) return y * sc;
  wk *= w;
  y += c6 * wk;
  return y * sc;
}

/* lambda.c:101-191: correctly rounded Lambda(i) for i < 256, series beyond.
 * The table is rebuilt here from Lambda(0) = sqrt(pi) and the exact ratio
 * Lambda(i+1) = Lambda(i) (i+1/2)/(i+1) in extended precision. */
static double orc_lamint[256];
static int orc_lamint_ready = 0;

static void orc_build_lamint(void) {
  if (orc_lamint_ready) return;
  long double v = sqrtl(3.14159265358979323846264338327950288L);
  for (int i = 0; i < 256; i++) {
    orc_lamint[i] = (double)v;
    v = v * ((long double)i + 0.5L) / ((long double)i + 1.0L);
  }
  orc_lamint_ready = 1;
}

double orc_LambdaI(size_t z) {
  if (z > 255) return orc_Lambda((double)z);
  orc_build_lamint();
  return orc_lamint[z];
}

/* ---------------------------------------------------------------------------
 * Binomial transfer matrix (leg2cheb.c:6-123 tables BMe/BMeT, generated by
 * src/python/binommat.py:33-61): entry (i, j) is the coefficient of T_j(x) in
 * T_i((x-1)/2).  Built by the three-term recurrence in the Chebyshev basis;
 * every intermediate value is a short dyadic rational, so doubles are exact.
 * ------------------------------------------------------------------------- */
static void orc_binomial(double *B, double *BT) {
  double C[ORC_M][ORC_M];
  double prev[ORC_M + 1], cur[ORC_M + 1], nxt[ORC_M + 1], xc[ORC_M + 2];
  memset(C, 0, sizeof(C));
  memset(prev, 0, sizeof(prev));
  memset(cur, 0, sizeof(cur));
  prev[0] = 1.0;           /* T_0(y) = 1            */
  cur[0] = -0.5;           /* T_1(y) = y = x/2 - 1/2 */
  cur[1] = 0.5;
  C[0][0] = 1.0;
  C[1][0] = -0.5;
  C[1][1] = 0.5;
  for (int i = 1; i + 1 < ORC_M; i++) {
    /* x * cur in the Chebyshev basis: x T_0 = T_1, x T_j = (T_{j+1} + T_{j-1})/2 */
    memset(xc, 0, sizeof(xc));
    for (int j = 0; j <= i; j++) {
      if (j == 0) {
        xc[1] += cur[0];
      } else {
        xc[j + 1] += 0.5 * cur[j];
        xc[j - 1] += 0.5 * cur[j];
      }
    }
    /* T_{i+1}(y) = 2 y T_i(y) - T_{i-1}(y), 2y = x - 1 */
    memset(nxt, 0, sizeof(nxt));
    for (int j = 0; j <= i + 1; j++) nxt[j] = xc[j] - cur[j] - prev[j];
    for (int j = 0; j <= i + 1; j++) C[i + 1][j] = nxt[j];
    memcpy(prev, cur, sizeof(cur));
    memcpy(cur, nxt, sizeof(cur));
  }
  size_t k = 0;
  for (int i = 0; i < ORC_M; i++)
    for (int j = 0; j <= i; j++) B[k++] = C[i][j];
  k = 0;
  for (int i = 0; i < ORC_M; i++)
    for (int j = i; j < ORC_M; j++) BT[k++] = C[j][i];
}

/* Tree bookkeeping, leg2cheb.c:125-150 */
static size_t nblocks(size_t level) { return ((size_t)2 << level) - 1; }
static size_t total_blocks(size_t L) { return ((size_t)2 << L) - (L + 2); }
static size_t level_h(size_t level, size_t L) { return (size_t)1 << (L - level - 1); }

/* leg2cheb.c:758-818: Lambda tables for the direct/near-field sums */
static void orc_lambda_tables(orc_plan *p, size_t N, size_t dirs) {
  double *a = (double *)malloc((N ? N : 1) * sizeof(double));
  const size_t head = N < 256 ? N : 256;
  for (size_t i = 0; i < head; i++) a[i] = orc_LambdaI(i);
  for (size_t i = head; i < N; i += 8) {
    a[i] = orc_LambdaI(i);
    const size_t stop = i + 8 < N ? i + 8 : N;
    for (size_t j = i + 1; j < stop; j++) a[j] = a[j - 1] - 0.5 * a[j - 1] / j;
  }
  p->a = a;
  p->an = p->dn = NULL;
  if (dirs == ORC_C2L || dirs == ORC_BOTH) {
    double *an = (double *)malloc((N ? N : 1) * sizeof(double));
    double *dn = (double *)malloc(((N + 1) / 2 ? (N + 1) / 2 : 1) * sizeof(double));
    if (N > 0) an[0] = 1.12837916709551257390; /* 2/sqrt(pi) */
    for (size_t i = 1; i < N; i++) an[i] = 1 / (a[i] * (2 * i * i + i));
    if ((N + 1) / 2 > 0) dn[0] = 0;
    for (size_t i = 1; i < (N + 1) / 2; i++) dn[i] = a[i - 1] / (2 * i);
    p->an = an;
    p->dn = dn;
  }
}

/* 2D DCT-II of an 18x18 sample grid scaled to Chebyshev coefficients:
 * out = (4/M^2) C F C^T with C[k][n] = cos(pi k (n+1/2)/M), then row 0 and
 * column 0 halved (dct.c:582-598, the same transform the reference computes
 * with its radix-2/3 factorisation; here as plain cosine sums). */
static void orc_dct2(const double *F, double *out) {
  static double cs[ORC_M][ORC_M];
  static int ready = 0;
  if (!ready) {
#pragma omp critical(orc_dct_table)
    {
      if (!ready) {
        for (int k = 0; k < ORC_M; k++)
          for (int n = 0; n < ORC_M; n++)
            cs[k][n] = cos(3.14159265358979323846 * k * (n + 0.5) / ORC_M);
        ready = 1;
      }
    }
  }
  double tmp[ORC_M][ORC_M];
  for (int i = 0; i < ORC_M; i++)
    for (int k = 0; k < ORC_M; k++) {
      double acc = 0;
      for (int n = 0; n < ORC_M; n++) acc += F[i * ORC_M + n] * cs[k][n];
      tmp[i][k] = acc;
    }
  for (int k1 = 0; k1 < ORC_M; k1++)
    for (int k2 = 0; k2 < ORC_M; k2++) {
      double acc = 0;
      for (int i = 0; i < ORC_M; i++) acc += cs[k1][i] * tmp[i][k2];
      out[k1 * ORC_M + k2] = acc * (1.0 / 81.0);
    }
  for (int i = 0; i < ORC_M; i++) {
    out[i] *= 0.5;
    out[i * ORC_M] *= 0.5;
  }
}

/* leg2cheb.c:924-995: far-field blocks.  For level l, block b, (q,p) in
 * {(0,0),(1,0),(1,1)} sample the kernel on the 18x18 Chebyshev grid
 *   L2C: Lambda((y-x)/2) Lambda((x+y)/2)
 *   C2L: 2 Lambda((y-x)/2) / (Lambda((x+y)/2) (x+y) (x+y+1) (x-y+1))
 * with x = x0 + h xj[i], y = y0 + h xj[j], and convert with orc_dct2.  The
 * shift-invariant factor Lambda((y-x)/2) is evaluated once per level (block 0)
 * and filled persymmetrically; Lambda((x+y)/2) is filled symmetrically, as in
 * the reference, so both ports round identically. */
static void orc_assemble(orc_plan *p) {
  const size_t L = p->L, s = p->s;
  double xj[ORC_M];
  for (int i = 0; i < ORC_M; i++) xj[i] = cos((i + 0.5) * 3.14159265358979323846 / ORC_M);
  size_t ndir = 0, dlist[2];
  if (p->dirs == ORC_L2C || p->dirs == ORC_BOTH) dlist[ndir++] = ORC_L2C;
  if (p->dirs == ORC_C2L || p->dirs == ORC_BOTH) dlist[ndir++] = ORC_C2L;
  size_t kk = 0;
  for (size_t level = 0; level < L; level++) {
    const size_t h = s * level_h(level, L);
    double xjh[ORC_M];
    for (int k = 0; k < ORC_M; k++) xjh[k] = xj[k] * h;
    /* Lambda((y-x)/2) for q-p = 0 and 1, from block 0 with p = 0 */
    double f0[2][ORC_MM];
    for (size_t q = 0; q < 2; q++) {
      const size_t i0 = 0, j0 = 2 * s * level_h(level, L);
      const double x0 = (double)(2 * i0 + h), y0 = (double)(2 * (j0 + q * h) + h);
      for (int i = 0; i < ORC_M; i++)
        for (int j = 0; j < ORC_M - i; j++) {
          const double x = x0 + xjh[i], y = y0 + xjh[j];
          const double m0 = orc_Lambda((y - x) / 2);
          f0[q][i * ORC_M + j] = m0;
          f0[q][(ORC_M - 1 - j) * ORC_M + (ORC_M - 1 - i)] = m0;
        }
    }
    const size_t nb = nblocks(level);
#pragma omp parallel for schedule(static)
    for (size_t block = 0; block < nb; block++) {
      const size_t i0 = 2 * block * s * level_h(level, L);
      const size_t j0 = i0 + 2 * s * level_h(level, L);
      size_t r = 0;
      for (size_t q = 0; q < 2; q++) {
        const double y0 = (double)(2 * (j0 + q * h) + h);
        for (size_t pp = 0; pp <= q; pp++, r++) {
          const double x0 = (double)(2 * (i0 + pp * h) + h);
          double f1[ORC_MM], F[ORC_MM];
          for (int i = 0; i < ORC_M; i++)
            for (int j = i; j < ORC_M; j++) {
              const double x = x0 + xjh[i], y = y0 + xjh[j];
              const double m1 = orc_Lambda((x + y) / 2);
              f1[i * ORC_M + j] = m1;
              f1[j * ORC_M + i] = m1;
            }
          const double *fpq = f0[q - pp];
          for (size_t di = 0; di < ndir; di++) {
            const size_t dir = dlist[di];
            for (int i = 0; i < ORC_M; i++)
              for (int j = 0; j < ORC_M; j++) {
                const int ix = i * ORC_M + j;
                const double x = x0 + xjh[i], y = y0 + xjh[j];
                if (dir == ORC_L2C)
                  F[ix] = fpq[ix] * f1[ix];
                else
                  F[ix] = 2 * (fpq[ix] / (f1[ix] * (x + y) * (x + y + 1) * (x - y + 1)));
              }
            double *dst = &p->A[dir][(kk + 3 * block + r) * ORC_MM];
            if (p->lagrange) /* nodal: the samples themselves (leg2cheb.c:938, 973) */
              memcpy(dst, F, sizeof(F));
            else
              orc_dct2(F, dst);
          }
        }
      }
    }
    kk += 3 * nb;
  }
}

/* leg2cheb.c:621-648: T_j(-1 + i/s) for i < 2s, rows split even | odd */
static void orc_vandermonde(orc_plan *p) {
  const size_t s = p->s;
  double *T = (double *)malloc(2 * s * ORC_M * sizeof(double));
  double row[ORC_M];
  for (size_t i = 0; i < 2 * s; i++) {
    const double x = -1 + (double)i / (double)s;
    const double x2 = 2 * x;
    row[0] = 1;
    row[1] = x;
    for (int j = 2; j < ORC_M; j++) row[j] = row[j - 1] * x2 - row[j - 2];
    double *dst = (i % 2 == 0) ? &T[(i / 2) * ORC_M] : &T[(s + i / 2) * ORC_M];
    memcpy(dst, row, sizeof(row));
  }
  p->T = T;
}

/* Nodal form, leg2cheb.c:997-1031: barycentric Lagrange weights from the M
 * Chebyshev points x_j = cos((j + 1/2) pi / M) (weights w_j = (-1)^j
 * sin((j + 1/2) pi / M)) to the 2s equispaced points -1 + i/s, each row divided
 * by its sum; rows split even | odd as in the modal T. */
static void orc_lagrange_T(orc_plan *p) {
  const size_t s = p->s;
  const double pi = 3.14159265358979323846;
  double xj[ORC_M], wj[ORC_M];
  for (int j = 0; j < ORC_M; j++) {
    xj[j] = cos((j + 0.5) * pi / ORC_M);
    wj[j] = ((j % 2 == 0) ? 1 : -1) * sin((j + 0.5) * pi / ORC_M);
  }
  double *T = (double *)malloc(2 * s * ORC_M * sizeof(double));
  for (size_t i = 0; i < s; i++) {
    const double xe = -1 + (double)(2 * i) / (double)s, xo = -1 + (double)(2 * i + 1) / (double)s;
    double sume = 0.0, sumo = 0.0;
    for (int j = 0; j < ORC_M; j++) {
      const double se = wj[j] / (xe - xj[j]), so = wj[j] / (xo - xj[j]);
      T[i * ORC_M + j] = se;
      T[(s + i) * ORC_M + j] = so;
      sume += se;
      sumo += so;
    }
    for (int j = 0; j < ORC_M; j++) {
      T[i * ORC_M + j] /= sume;
      T[(s + i) * ORC_M + j] /= sumo;
    }
  }
  p->T = T;
}

/* Nodal transfer matrices, leg2cheb.c:1076-1100: B_c[i][j] = l_j((x_i - 1)/2)
 * (child c = 0) and l_j((x_i + 1)/2) (c = 1), l_j the barycentric Lagrange
 * basis of the Chebyshev points, rows normalised by their sums. */
static void orc_lagrange_B(double *B) {
  const double pi = 3.14159265358979323846;
  double xj[ORC_M], wj[ORC_M];
  for (int j = 0; j < ORC_M; j++) {
    xj[j] = cos((j + 0.5) * pi / ORC_M);
    wj[j] = ((j % 2 == 0) ? 1 : -1) * sin((j + 0.5) * pi / ORC_M);
  }
  for (int i = 0; i < ORC_M; i++) {
    const double x0 = (xj[i] - 1) / 2, x1 = (xj[i] + 1) / 2;
    double sum0 = 0.0, sum1 = 0.0;
    for (int j = 0; j < ORC_M; j++) {
      const double s0 = wj[j] / (x0 - xj[j]), s1 = wj[j] / (x1 - xj[j]);
      B[i * ORC_M + j] = s0;
      B[ORC_MM + i * ORC_M + j] = s1;
      sum0 += s0;
      sum1 += s1;
    }
    for (int j = 0; j < ORC_M; j++) {
      B[i * ORC_M + j] /= sum0;
      B[ORC_MM + i * ORC_M + j] /= sum1;
    }
  }
}

orc_plan *orc_create(size_t N, size_t maxs, size_t dirs) {
  return orc_create_ex(N, maxs, dirs, 0);
}

orc_plan *orc_create_ex(size_t N, size_t maxs, size_t dirs, size_t lagrange) {
  orc_plan *p = (orc_plan *)calloc(1, sizeof(orc_plan));
  p->N = N;
  p->dirs = dirs;
  p->lagrange = lagrange ? 1 : 0;
  orc_binomial(p->B, p->BT);
  orc_lagrange_B(p->LB);
  /* leg2cheb.c:860-871 */
  const int L = (int)ceil(log2((double)N / (double)maxs)) - 2;
  if (L < 1) {
    p->L = 0;
    p->Nn = N;
    orc_lambda_tables(p, N, dirs);
    return p;
  }
  p->L = (size_t)L;
  p->s = (size_t)ceil((double)N / pow(2, L + 2));
  p->Nn = p->s * ((size_t)1 << (L + 2));
  p->Nb = total_blocks(p->L);
  orc_lambda_tables(p, N, dirs);
  for (size_t d = 0; d < 2; d++) {
    if (dirs == d || dirs == ORC_BOTH)
      p->A[d] = (double *)malloc(3 * p->Nb * ORC_MM * sizeof(double));
  }
  orc_assemble(p);
  if (p->lagrange)
    orc_lagrange_T(p);
  else
    orc_vandermonde(p);
  return p;
}

void orc_free(orc_plan *p) {
  if (!p) return;
  free(p->a);
  free(p->an);
  free(p->dn);
  free(p->A[0]);
  free(p->A[1]);
  free(p->T);
  free(p);
}

void orc_plan_info(const orc_plan *p, size_t *info) {
  info[0] = p->N;
  info[1] = p->L;
  info[2] = p->s;
  info[3] = p->Nn;
  info[4] = p->Nb;
  info[5] = ORC_M;
}
const double *orc_plan_A(const orc_plan *p, size_t d) { return d < 2 ? p->A[d] : NULL; }
const double *orc_plan_T(const orc_plan *p) { return p->T; }
const double *orc_plan_lambda(const orc_plan *p) { return p->a; }
const double *orc_plan_B(const orc_plan *p) { return p->lagrange ? p->LB : p->B; }
const double *orc_plan_BT(const orc_plan *p) { return p->lagrange ? NULL : p->BT; }

/* ---------------------------------------------------------------------------
 * Direct O(N^2) transform, leg2cheb.c:152-234 (used when L < 1).  Reproduces
 * the reference's contract exactly: out[0..N) is zeroed contiguously, the L2C
 * input is read contiguously whatever the stride, and nothing is scaled except
 * b[0] /= 2 (L2C) or the (i + 1/2) factor (C2L).
 * ------------------------------------------------------------------------- */
static size_t orc_direct(const double *u, double *b, const orc_plan *p, size_t dir,
                         size_t stride) {
  const size_t N = p->N;
  const double rpi = 1.77245385090551602e0; /* sqrt(pi) */
  size_t flops = N;
  for (size_t i = 0; i < N; i++) b[i] = 0.0;
  if (dir == ORC_L2C) {
    const double *a = p->a;
    for (size_t n = 0; n < N; n += 2) {
      const double a0 = a[n / 2] * 0.63661977236758134308; /* 2/pi */
      for (size_t i = 0; i < N - n; i++) b[i * stride] += a0 * a[n / 2 + i] * u[n + i];
      flops += 3 * (N - n);
    }
    b[0] /= 2;
    flops += N;
  } else {
    const double *an = p->an, *dn = p->dn;
    double *v = (double *)malloc((N ? N : 1) * sizeof(double));
    v[0] = u[0];
    for (size_t i = 1; i < N; i++) v[i] = u[i * stride] * i;
    for (size_t n = 0; n < N; n++) b[n * stride] = rpi * v[n] * an[n];
    for (size_t n = 2; n < N; n += 2) {
      for (size_t i = 0; i < N - n; i++) b[i * stride] -= dn[n / 2] * an[n / 2 + i] * v[n + i];
      flops += 3 * (N - n);
    }
    for (size_t i = 0; i < N; i++) b[i * stride] *= (i + 0.5);
    flops += N;
    free(v);
  }
  return flops;
}

/* Near field of L2C, leg2cheb.c:236-376: for block i0 = b h (h = 2s), even
 * n < 4s, out[i0+i] += Lambda(n/2) Lambda(i0+n/2+i) u[i0+i+n] for i + n < 2h;
 * the last block takes every remaining source; then out *= 2/pi, out[0] /= 2. */
static size_t orc_near_l2c(const double *u, double *out, const orc_plan *p, size_t st) {
  const size_t s = p->s, N = p->N, h = 2 * s, nL = N / h;
  const double *a = p->a;
  size_t flops = 0;
#pragma omp parallel for reduction(+ : flops) schedule(static)
  for (size_t blk = 0; blk < nL - 1; blk++) {
    const size_t i0 = blk * h;
    for (size_t n = 0; n < 4 * s; n += 2) {
      const double a0 = a[n / 2];
      const double *ap = &a[i0 + n / 2];
      const size_t cnt = n < h ? h : 2 * h - n;
      for (size_t i = 0; i < cnt; i++)
        out[(i0 + i) * st] += a0 * ap[i] * u[(i0 + n + i) * st];
      flops += 3 * cnt;
    }
  }
  const size_t i0 = (nL - 1) * h;
  for (size_t n = 0; 2 * n + i0 < N; n++) {
    const double a0 = a[n];
    const size_t cnt = N - (2 * n + i0);
    for (size_t i = 0; i < cnt; i++)
      out[(i0 + i) * st] += a0 * a[n + i0 + i] * u[(i0 + 2 * n + i) * st];
    flops += 3 * cnt;
  }
  for (size_t i = 0; i < N; i++) out[i * st] *= 0.63661977236758134308;
  out[0] *= 0.5;
  return flops + N;
}

/* Near field of C2L, leg2cheb.c:378-535 (the live, non-precomputed branch):
 * diagonal sqrt(pi) v an, minus dn[n/2] v[i0+i+n] an[i0+n/2+i] over the band,
 * then out *= (i + 1/2).  v is the premultiplied contiguous copy of the input. */
static size_t orc_near_c2l(const double *v, double *out, const orc_plan *p, size_t st) {
  const size_t s = p->s, N = p->N, h = 2 * s, nL = N / h;
  const double *an = p->an, *dn = p->dn;
  const double rpi = 1.77245385090551602729816e0;
  size_t flops = 3 * N;
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < N; i++) out[i * st] += rpi * v[i] * an[i];
#pragma omp parallel for reduction(+ : flops) schedule(static)
  for (size_t blk = 0; blk < nL - 1; blk++) {
    const size_t i0 = blk * h;
    for (size_t n = 2; n < 4 * s; n += 2) {
      const double d0 = dn[n / 2];
      const size_t cnt = n < h ? h : 2 * h - n;
      for (size_t i = 0; i < cnt; i++)
        out[(i0 + i) * st] -= d0 * v[i0 + n + i] * an[i0 + n / 2 + i];
      flops += 3 * cnt;
    }
  }
  const size_t i0 = (nL - 1) * h;
  for (size_t n = 1; n < N - i0; n++) {
    for (size_t i = i0; i + 2 * n < N; i++)
      out[i * st] -= dn[n] * an[i + n] * v[i + 2 * n];
    flops += (N - (2 * n + i0)) * 3;
  }
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < N; i++) out[i * st] *= (i + 0.5);
  return flops + 2 * N;
}

size_t orc_directM(const double *in, double *out, orc_plan *p, size_t stride) {
  if (p->L == 0) return 0;
  return orc_near_l2c(in, out, p, stride);
}

size_t orc_directL(const double *v, double *out, orc_plan *p, size_t stride) {
  if (p->L == 0 || p->an == NULL) return 0;
  return orc_near_c2l(v, out, p, stride);
}

/* Lower compact triangular product with the +/- parity combination of two
 * children, leg2cheb.c:537-602 (M even): z+ = x0 + S x1, z- = x0 - S x1 with
 * S = diag(1,-1,1,...); b[i] = sum_j B[i][j] z+[j] (i even) or z-[j] (i odd). */
static void orc_up(const double *B, const double *x, double *b) {
  double zp[ORC_M], zm[ORC_M];
  for (int i = 0; i < ORC_M; i += 2) {
    zp[i] = x[i] + x[ORC_M + i];
    zm[i] = x[i] - x[ORC_M + i];
    zp[i + 1] = x[i + 1] - x[ORC_M + i + 1];
    zm[i + 1] = x[i + 1] + x[ORC_M + i + 1];
  }
  size_t k = 0;
  for (int i = 0; i < ORC_M; i++) {
    const double *z = (i % 2 == 0) ? zp : zm;
    double acc = B[k++] * z[0];
    for (int j = 1; j <= i; j++) acc += B[k++] * z[j];
    b[i] = acc;
  }
}

/* Upper compact triangular product into two children, leg2cheb.c:603-618:
 * se/so collect the columns of equal/opposite parity to the row;
 * child0 += se + so, child1 += se - so. */
static void orc_down(const double *BT, const double *x, double *b) {
  size_t k = 0;
  for (int i = 0; i < ORC_M; i++) {
    double se = 0.0, so = 0.0;
    int j = i;
    for (; j < ORC_M - 1; j += 2) {
      se += BT[k++] * x[j];
      so += BT[k++] * x[j + 1];
    }
    if ((i + ORC_M) % 2 == 1) se += BT[k++] * x[j];
    b[i] += se + so;
    b[ORC_M + i] += se - so;
  }
}

/* Nodal upward product, leg2cheb.c:1409-1412 (two dgemv, CblasTrans):
 * b[j] = sum_i B0[i][j] x0[i] + sum_i B1[i][j] x1[i]. */
static void orc_up_nodal(const double *LB, const double *x, double *b) {
  for (int j = 0; j < ORC_M; j++) {
    double acc = 0.0;
    for (int i = 0; i < ORC_M; i++) acc += LB[i * ORC_M + j] * x[i];
    b[j] = acc;
  }
  for (int j = 0; j < ORC_M; j++) {
    double acc = 0.0;
    for (int i = 0; i < ORC_M; i++) acc += LB[ORC_MM + i * ORC_M + j] * x[ORC_M + i];
    b[j] += acc;
  }
}

/* Nodal downward product, leg2cheb.c:1457-1460 (two dgemv, beta = 1):
 * child0[i] += sum_j B0[i][j] x[j], child1[i] += sum_j B1[i][j] x[j]. */
static void orc_down_nodal(const double *LB, const double *x, double *b) {
  for (int c = 0; c < 2; c++)
    for (int i = 0; i < ORC_M; i++) {
      double acc = 0.0;
      for (int j = 0; j < ORC_M; j++) acc += LB[c * ORC_MM + i * ORC_M + j] * x[j];
      b[c * ORC_M + i] += acc;
    }
}

/* One FMM transform, leg2cheb.c:1299-1500. */
size_t orc_execute(const double *in, double *out, orc_plan *p, size_t dir, size_t stride) {
  if (dir > 1) return 0;
  if (dir == ORC_C2L && p->an == NULL) return 0;
  if (p->L == 0) return orc_direct(in, out, p, dir, stride);
  if (p->A[dir] == NULL) return 0;
  const size_t N = p->N, L = p->L, s = p->s, Nn = p->Nn, Nb = p->Nb, M = ORC_M;
  const double *A = p->A[dir];
  size_t flops = 0;

  /* C2L works on v_j = j u_j (j >= 2), leg2cheb.c:1325-1335 */
  double *v = NULL;
  if (dir == ORC_C2L) {
    v = (double *)malloc(N * sizeof(double));
    v[0] = in[0];
    v[1] = in[stride];
    for (size_t i = 2; i < N; i++) v[i] = in[i * stride] * i;
  }
  double *ia = (double *)malloc(Nn / 2 * sizeof(double));
  double *oa = (double *)malloc(Nn / 2 * sizeof(double));
  double *wk = (double *)malloc(Nb * 2 * M * sizeof(double));
  double *ck = (double *)malloc(Nb * 2 * M * sizeof(double));
  size_t *lvl = (size_t *)malloc(L * sizeof(size_t)); /* level offsets in wk/ck */
  lvl[0] = 0;
  for (size_t l = 1; l < L; l++) lvl[l] = lvl[l - 1] + nblocks(l - 1) * 2 * M;
  const size_t K = nblocks(L - 1) * 2;

  for (size_t odd = 0; odd < 2; odd++) {
    memset(oa, 0, Nn / 2 * sizeof(double));
    memset(wk, 0, Nb * 2 * M * sizeof(double));
    memset(ck, 0, Nb * 2 * M * sizeof(double));
    /* parity split with zero padding, leg2cheb.c:1350-1376 */
    const size_t cnt = N / 2 + (N % 2) * (1 - odd);
    for (size_t i = 0; i < cnt; i++)
      ia[i] = (dir == ORC_C2L) ? v[2 * i + odd] : in[(2 * i + odd) * stride];
    for (size_t i = cnt; i < Nn / 2; i++) ia[i] = 0;

    /* step 1: leaf coefficients, wk[L-1] (K x M) = ia[2s:] (K x s) T_odd (s x M) */
    const double *To = &p->T[odd * s * M];
    double *wl = &wk[lvl[L - 1]];
#ifdef ORC_CBLAS
#pragma omp parallel
    {
      size_t r0 = 0, r1 = K;
#ifdef _OPENMP
      const size_t nt = (size_t)omp_get_num_threads(), id = (size_t)omp_get_thread_num();
      r0 = K * id / nt;
      r1 = K * (id + 1) / nt;
#endif
      if (r1 > r0)
        scipy_cblas_dgemm(OrcRowMajor, OrcNoTrans, OrcNoTrans, (int)(r1 - r0), (int)M, (int)s,
                          1.0, &ia[2 * s + r0 * s], (int)s, To, (int)M, 0.0, wl + r0 * M, (int)M);
    }
#else
#pragma omp parallel for schedule(static)
    for (size_t r = 0; r < K; r++)
      for (size_t m = 0; m < M; m++) {
        double acc = 0;
        for (size_t i = 0; i < s; i++) acc += ia[2 * s + r * s + i] * To[i * M + m];
        wl[r * M + m] = acc;
      }
#endif
    flops += 2 * K * s * M;

    /* step 2: upward transfer, leg2cheb.c:1385-1399 (modal) and 1401-1416
     * (nodal: parent = B0^T child0 + B1^T child1) */
    for (size_t level = L; level-- > 1;) {
      double *w1 = &wk[lvl[level - 1]];
      const double *w2 = &wk[lvl[level]];
#pragma omp parallel for schedule(static)
      for (size_t block = 1; block < nblocks(level); block++) {
        const size_t b0 = (block - 1) / 2, q0 = (block - 1) % 2;
        if (p->lagrange)
          orc_up_nodal(p->LB, &w2[block * 2 * M], &w1[(b0 * 2 + q0) * M]);
        else
          orc_up(p->B, &w2[block * 2 * M], &w1[(b0 * 2 + q0) * M]);
      }
      flops += (nblocks(level) - 1) * M * M * (p->lagrange ? 4 : 1);
    }

    /* step 3: far-field blocks, leg2cheb.c:1419-1435 */
    for (size_t level = 0; level < L; level++) {
      const double *ap = &A[3 * (total_blocks(level)) * M * M];
      double *cp = &ck[lvl[level]];
      const double *wq = &wk[lvl[level]];
#pragma omp parallel for schedule(static)
      for (size_t block = 0; block < nblocks(level); block++) {
        const double *A0 = &ap[(3 * block) * M * M], *A1 = A0 + M * M, *A2 = A1 + M * M;
        const double *w0 = &wq[block * 2 * M], *w1 = w0 + M;
        double *c0 = &cp[block * 2 * M], *c1 = c0 + M;
        for (size_t i = 0; i < M; i++) {
          double t0 = 0, t1 = 0, t2 = 0;
          for (size_t j = 0; j < M; j++) {
            t0 += A0[i * M + j] * w0[j];
            t1 += A1[i * M + j] * w1[j];
            t2 += A2[i * M + j] * w1[j];
          }
          c0[i] = t0 + t1;
          c1[i] = t2;
        }
      }
    }
    flops += 3 * Nb * 2 * M * M;

    /* step 4: downward transfer, leg2cheb.c:1437-1448 (modal) and 1450-1464
     * (nodal: child_c += B_c parent) */
    for (size_t level = 0; level + 1 < L; level++) {
      const double *c0 = &ck[lvl[level]];
      double *c1 = &ck[lvl[level + 1]];
#pragma omp parallel for schedule(static)
      for (size_t block = 0; block < nblocks(level + 1) - 1; block++) {
        if (p->lagrange)
          orc_down_nodal(p->LB, &c0[block * M], &c1[block * 2 * M]);
        else
          orc_down(p->BT, &c0[block * M], &c1[block * 2 * M]);
      }
      flops += (nblocks(level + 1) - 1) * M * M * (p->lagrange ? 4 : 1);
    }

    /* step 5: back to leaf values and scatter, leg2cheb.c:1467-1483 */
    const double *cl = &ck[lvl[L - 1]];
#ifdef ORC_CBLAS
#pragma omp parallel
    {
      size_t r0 = 0, r1 = K;
#ifdef _OPENMP
      const size_t nt = (size_t)omp_get_num_threads(), id = (size_t)omp_get_thread_num();
      r0 = K * id / nt;
      r1 = K * (id + 1) / nt;
#endif
      if (r1 > r0)
        scipy_cblas_dgemm(OrcRowMajor, OrcNoTrans, OrcTrans, (int)(r1 - r0), (int)s, (int)M, 1.0,
                          cl + r0 * M, (int)M, To, (int)M, 0.0, oa + r0 * s, (int)s);
    }
#else
#pragma omp parallel for schedule(static)
    for (size_t r = 0; r < K; r++)
      for (size_t i = 0; i < s; i++) {
        double acc = 0;
        for (size_t m = 0; m < M; m++) acc += cl[r * M + m] * To[i * M + m];
        oa[r * s + i] = acc;
      }
#endif
    flops += 2 * K * s * M;
    for (size_t k = 0; k < cnt; k++) out[(2 * k + odd) * stride] += oa[k];
  }

  if (dir == ORC_L2C)
    flops += orc_near_l2c(in, out, p, stride);
  else
    flops += orc_near_c2l(v, out, p, stride);

  free(lvl);
  free(ia);
  free(oa);
  free(wk);
  free(ck);
  free(v);
  return flops;
}

/* Many independent transforms with one plan, one vector per OpenMP thread (the
 * per-call parallel loops of orc_execute then run single-threaded inside this
 * region).  The CPU harness for batched workloads; plan data is read-only and
 * every call allocates its own work arrays, so concurrent calls are safe. */
size_t orc_execute_batch(const double *in, double *out, orc_plan *p, size_t direction,
                         size_t count, size_t dist, size_t stride) {
  size_t flops = 0;
#pragma omp parallel for reduction(+ : flops) schedule(dynamic, 1)
  for (size_t v = 0; v < count; v++)
    flops += orc_execute(in + v * dist, out + v * dist, p, direction, stride);
  return flops;
}

/* Ragged list: vector v of plans[v]->N coefficients at in + off[v], out + off[v],
 * one vector per OpenMP thread (CPU harness for ragged workloads). */
size_t orc_execute_ragged(const double *in, double *out, orc_plan **plans, const size_t *off,
                          size_t count, size_t direction) {
  size_t flops = 0;
#pragma omp parallel for reduction(+ : flops) schedule(dynamic, 1)
  for (size_t v = 0; v < count; v++)
    flops += orc_execute(in + off[v], out + off[v], plans[v], direction, 1);
  return flops;
}
