/* leg2cheb_host.c -- the reference's public C API (include/leg2cheb.h) on top
 * of the GPU implementation (include/l2c_cuda.h).
 *
 * Every transform runs on the GPU; this file only manages plans, mirrors the
 * reference's host-visible plan fields, and forwards calls.  There is no CPU
 * transform path: without a working CUDA device create_fmm() returns NULL and
 * execute() returns 0, with the reason in l2c_last_error().
 *
 * Compiled with -ffp-contract=off so the few host-side plan values (the
 * Vandermonde rows kept in fmm_plan->T) round exactly as the reference's. */
#include "../../include/leg2cheb.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/l2c_cuda.h"
#include "l2c_tables.h"

#define L2C_M 18

static __thread char host_err[512] = "";

static void herr(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(host_err, sizeof(host_err), fmt, ap);
  va_end(ap);
}

const char *l2c_last_error(void) {
  if (host_err[0]) return host_err;
  return l2c_gpu_last_error();
}

/* The exact binomial transfer tables (leg2cheb.c:6-123), exposed through
 * fmm_plan->B / ->BT as in the reference. */
static const double binom_lower[(L2C_M * L2C_M + L2C_M) / 2] = L2C_BINOM_LOWER_INIT;
static const double binom_upper[(L2C_M * L2C_M + L2C_M) / 2] = L2C_BINOM_UPPER_INIT;

/* ------------------------------------------------------------------------ */
/* Tree bookkeeping, leg2cheb.c:125-150                                      */
/* ------------------------------------------------------------------------ */
size_t get_number_of_blocks(const size_t level) { return ((size_t)2 << level) - 1; }
size_t get_h(const size_t level, const size_t L) { return (size_t)1 << (L - level - 1); }
size_t get_number_of_submatrices(const size_t level) { return 3 * get_number_of_blocks(level); }
size_t get_total_number_of_blocks(const size_t L) { return ((size_t)2 << L) - (L + 2); }
size_t get_total_number_of_submatrices(const size_t L) {
  return 3 * get_total_number_of_blocks(L);
}
void get_ij(size_t *ij, const size_t level, const size_t block, const size_t s, const size_t L) {
  const size_t h = get_h(level, L);
  ij[0] = 2 * block * s * h;
  ij[1] = ij[0] + 2 * s * h;
}

/* ------------------------------------------------------------------------ */
/* Lambda, lambda.c                                                          */
/* ------------------------------------------------------------------------ */
double Lambda(const double z) { return l2c_lambda(z); }
double LambdaI(const size_t z) { return l2c_lambda_int(z); }
void Lambdavec(const double *z, double *w, const size_t N) {
  for (size_t i = 0; i < N; i++) w[i] = l2c_lambda(z[i]);
}
/* Through log-gamma (lambda.c:20). */
double _Lambda0(const double z) { return exp(lgamma(z + 0.5) - lgamma(z + 1)); }
/* Second evaluation route (the reference's lambda.c:51-63 uses a Chebyshev fit):
 * step the argument up past 16 with the exact ratio and take the full seven-term
 * series there.  Agrees with Lambda() to within an ulp or two. */
double _LambdaE(const double z) {
  if (z < 16) return _LambdaE(z + 1) * (z + 1) / (z + 0.5);
  const double zp = z + 0.25, w = 1 / (zp * zp);
  const double c[7] = {L2C_LAMBDA_C0, L2C_LAMBDA_C1, L2C_LAMBDA_C2, L2C_LAMBDA_C3,
                       L2C_LAMBDA_C4, L2C_LAMBDA_C5, L2C_LAMBDA_C6};
  double y = c[6];
  for (int k = 5; k >= 0; k--) y = y * w + c[k];
  return y / sqrt(zp);
}

/* ------------------------------------------------------------------------ */
/* 18-point DCT-II helpers (dct.c).  out[k] = sum_n x[n] cos(pi k (n+1/2)/18). */
/* ------------------------------------------------------------------------ */
static double dct_table[L2C_M][L2C_M];
static int dct_ready = 0;
static void dct_init(void) {
  if (dct_ready) return;
  for (int k = 0; k < L2C_M; k++)
    for (int n = 0; n < L2C_M; n++)
      dct_table[k][n] = cos(3.14159265358979323846 * k * (n + 0.5) / L2C_M);
  dct_ready = 1;
}
static void dct_plain(const double *in, double *out, size_t st) {
  double x[L2C_M];
  dct_init();
  for (int n = 0; n < L2C_M; n++) x[n] = in[n * st];
  for (int k = 0; k < L2C_M; k++) {
    double acc = 0;
    for (int n = 0; n < L2C_M; n++) acc += x[n] * dct_table[k][n];
    out[k * st] = acc;
  }
}
void dct(double *input, double *output, size_t st) { dct_plain(input, output, st); }
void dct0(double *input, double *output, size_t st) { dct_plain(input, output, st); }
void dct_radix2(double *input, double *output, size_t st) { dct_plain(input, output, st); }
void dct_radix23(double *input, double *output, size_t st) { dct_plain(input, output, st); }
void dct_fft(double *input, double *output, size_t st) { dct_plain(input, output, st); }
/* 2D transform scaled to Chebyshev coefficients: (4/M^2) C F C^T, row 0 and
 * column 0 halved (dct.c:582-598). */
void dct2(double *input, double *output) {
  double tmp[L2C_M * L2C_M];
  for (int i = 0; i < L2C_M; i++) dct_plain(input + i * L2C_M, tmp + i * L2C_M, 1);
  for (int i = 0; i < L2C_M; i++) dct_plain(tmp + i, output + i, L2C_M);
  for (int i = 0; i < L2C_M * L2C_M; i++) output[i] *= 1.0 / 81.0;
  for (int i = 0; i < L2C_M; i++) {
    output[i] *= 0.5;
    output[i * L2C_M] *= 0.5;
  }
}
/* In-place forward 9-point DFT, X_k = sum_n x_n exp(-2 pi i k n / 9). */
static void dft9(double (*x)[2]) {
  double re[9], im[9];
  for (int k = 0; k < 9; k++) {
    double sr = 0, si = 0;
    for (int n = 0; n < 9; n++) {
      const double ang = -2.0 * 3.14159265358979323846 * (double)((k * n) % 9) / 9.0;
      sr += x[n][0] * cos(ang) - x[n][1] * sin(ang);
      si += x[n][0] * sin(ang) + x[n][1] * cos(ang);
    }
    re[k] = sr;
    im[k] = si;
  }
  for (int k = 0; k < 9; k++) {
    x[k][0] = re[k];
    x[k][1] = im[k];
  }
}
#if defined(L2C_HAVE_FFTW_TYPES)
void fft9c(fftw_complex *x) { dft9((double (*)[2])x); }
void fft9(fftw_complex *x) { dft9((double (*)[2])x); }
#else
void fft9c(double (*x)[2]) { dft9(x); }
void fft9(double (*x)[2]) { dft9(x); }
#endif

/* ------------------------------------------------------------------------ */
/* Compact triangular transfer products, leg2cheb.c:537-619 (any m).         */
/* lower: b[i] = sum_{j<=i} A[i][j] z_i[j], z_i[j] = x[j] +- x[m+j] with the  */
/*        sign + when i + j is even, - when odd;                             */
/* upper: se/so = sums over columns j >= i of equal/opposite parity to i,    */
/*        b[i] += se + so, b[m+i] += se - so.                                */
/* ------------------------------------------------------------------------ */
void matvectri(const double *A, const double *x, double *b, const size_t m, const bool upper) {
  if (!upper) {
    const double *row = A;
    for (size_t i = 0; i < m; i++) {
      double acc = 0.0;
      for (size_t j = 0; j <= i; j++) {
        const double z = ((i + j) % 2 == 0) ? x[j] + x[m + j] : x[j] - x[m + j];
        acc += row[j] * z;
      }
      b[i] = acc;
      row += i + 1;
    }
  } else {
    const double *row = A;
    for (size_t i = 0; i < m; i++) {
      double se = 0.0, so = 0.0;
      for (size_t j = i; j < m; j++) {
        if ((j - i) % 2 == 0)
          se += row[j - i] * x[j];
        else
          so += row[j - i] * x[j];
      }
      b[i] += se + so;
      b[m + i] += se - so;
      row += m - i;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Plans                                                                     */
/* ------------------------------------------------------------------------ */

/* Host copies of the Lambda tables (the reference's direct_plan fields). */
static int fill_host_tables(direct_plan *dp, l2c_gpu_plan *gp, size_t N, size_t direction) {
  dp->a = (double *)malloc((N ? N : 1) * sizeof(double));
  if (!dp->a || l2c_gpu_plan_copy(gp, 2, dp->a, N) != N) return 0;
  if (direction == C2L || direction == BOTH) {
    const size_t nd = (N + 1) / 2;
    dp->an = (double *)malloc((N ? N : 1) * sizeof(double));
    dp->dn = (double *)malloc((nd ? nd : 1) * sizeof(double));
    if (!dp->an || !dp->dn) return 0;
    if (l2c_gpu_plan_copy(gp, 3, dp->an, N) != N) return 0;
    if (nd && l2c_gpu_plan_copy(gp, 4, dp->dn, nd) != nd) return 0;
  }
  return 1;
}

direct_plan *create_direct(size_t N, size_t direction, const size_t precompute) {
  (void)precompute; /* the band weights are formed on the fly on the GPU */
  host_err[0] = 0;
  direct_plan *dp = (direct_plan *)calloc(1, sizeof(direct_plan));
  if (!dp) {
    herr("out of host memory");
    return NULL;
  }
  dp->direction = direction;
  dp->N = N;
  l2c_gpu_plan *gp = l2c_gpu_plan_create(N, 1, direction, L2C_PLAN_DIRECT_ONLY);
  if (!gp) {
    free(dp);
    return NULL;
  }
  dp->gpu = gp;
  if (!fill_host_tables(dp, gp, N, direction)) {
    free_direct(dp);
    herr("could not copy the Lambda tables to the host");
    return NULL;
  }
  return dp;
}

void free_direct(direct_plan *dp) {
  if (!dp) return;
  if (dp->gpu) l2c_gpu_plan_destroy((l2c_gpu_plan *)dp->gpu);
  free(dp->a);
  free(dp->an);
  free(dp->dn);
  free(dp->lf);
  free(dp->lb);
  free(dp);
}

size_t direct(const double *input_array, double *output_array, direct_plan *dplan,
              size_t direction, size_t stride) {
  host_err[0] = 0;
  if (!dplan) {
    herr("null plan");
    return 0;
  }
  if (!dplan->gpu) {
    /* the direct_plan inside an FMM plan gets its O(N^2) GPU plan on first use */
    dplan->gpu = l2c_gpu_plan_create(dplan->N, 1, dplan->direction, L2C_PLAN_DIRECT_ONLY);
    if (!dplan->gpu) return 0;
  }
  return l2c_gpu_execute((l2c_gpu_plan *)dplan->gpu, input_array, output_array, direction, 1, 0,
                         stride, 0);
}

static void vandermonde_host(double *T, size_t s) {
  for (size_t i = 0; i < 2 * s; i++) {
    double row[L2C_M];
    const double xv = -1 + (double)i / (double)s;
    const double x2 = 2 * xv;
    row[0] = 1;
    row[1] = xv;
    for (int j = 2; j < L2C_M; j++) row[j] = row[j - 1] * x2 - row[j - 2];
    const size_t r = (i % 2 == 0) ? i / 2 : s + i / 2;
    memcpy(&T[r * L2C_M], row, sizeof(row));
  }
}

fmm_plan *create_fmm(const size_t N, const size_t maxs, const size_t M, const size_t direction,
                     const size_t lagrange, const size_t precompute, const size_t v) {
  return create_fmm_ex(N, maxs, M, direction, lagrange, precompute, v, 0);
}

fmm_plan *create_fmm_ex(const size_t N, const size_t maxs, const size_t M, const size_t direction,
                        const size_t lagrange, const size_t precompute, const size_t v,
                        unsigned flags) {
  host_err[0] = 0;
  if (M != L2C_M) {
    herr("only M = 18 is implemented (got M = %zu)", M);
    return NULL;
  }
  if (lagrange > 1) {
    herr("lagrange must be 0 (modal) or 1 (nodal)");
    return NULL;
  }
  if (direction > 2) {
    herr("direction must be 0 (L2C), 1 (C2L) or 2 (both)");
    return NULL;
  }
  fmm_plan *p = (fmm_plan *)calloc(1, sizeof(fmm_plan));
  if (!p) {
    herr("out of host memory");
    return NULL;
  }
  p->A = (double **)calloc(2, sizeof(double *));
  p->direction = direction;
  p->lagrange = lagrange;
  p->M = M;
  p->N = N;
  size_t s = 0, Nn = N;
  const size_t L = l2c_geometry(N, maxs, &s, &Nn);
  unsigned gflags = precompute ? L2C_PLAN_PRECOMPUTE_NEAR : 0;
  if (flags & L2C_FMM_MIXED) gflags |= L2C_PLAN_MIXED;
  if (lagrange == 1) gflags |= L2C_PLAN_NODAL;
  l2c_gpu_plan *gp = l2c_gpu_plan_create(N, maxs, direction, gflags);
  if (!gp) {
    free(p->A);
    free(p);
    return NULL;
  }
  p->gpu = gp;
  p->dplan = (direct_plan *)calloc(1, sizeof(direct_plan));
  p->dplan->N = N;
  p->dplan->direction = direction;
  if (!fill_host_tables(p->dplan, gp, N, direction)) {
    free_fmm(p);
    herr("could not copy the Lambda tables to the host");
    return NULL;
  }
  if (L == 0) {
    if (v > 1) printf("Levels < 1. Using only direct method\n");
    p->Nn = N;
    p->L = 0;
    return p;
  }
  p->L = L;
  p->s = s;
  p->Nn = Nn;
  if (v > 1) {
    printf("N %zu\n", N);
    printf("Num levels %zu\n", L);
    printf("Num submatrices %zu\n", get_total_number_of_submatrices(L));
    printf("Num blocks %zu\n", get_total_number_of_blocks(L));
    printf("Given max s %zu \n", maxs);
    printf("Computed s %zu \n", s);
    printf("Computed N %zu\n", Nn);
    printf("Lagrange %zu\n", lagrange);
    printf("Precomputed matrix entries %zu\n", precompute);
    printf("Using exact binomial matrix\n");
  }
  /* host mirrors of the plan fields the reference exposes (leg2cheb.c:1195-1211) */
  p->T = (double *)malloc(2 * s * L2C_M * sizeof(double));
  if (lagrange == 1) {
    /* nodal: T and B0 | B1 as the device plan built them; no BT (leg2cheb.c:1076-1100) */
    p->B = (double *)malloc(2 * L2C_M * L2C_M * sizeof(double));
    if (!p->T || !p->B || l2c_gpu_plan_copy(gp, 5, p->T, 2 * s * L2C_M) != 2 * s * L2C_M ||
        l2c_gpu_plan_copy(gp, 6, p->B, 2 * L2C_M * L2C_M) != 2 * L2C_M * L2C_M) {
      free_fmm(p);
      herr("could not copy the nodal plan tables to the host");
      return NULL;
    }
    p->BT = NULL;
  } else {
    vandermonde_host(p->T, s);
    p->B = (double *)binom_lower;
    p->BT = (double *)binom_upper;
  }
  const size_t Nb = get_total_number_of_blocks(L);
  p->ia = (double *)calloc(Nn / 2, sizeof(double));
  p->oa = (double *)calloc(Nn / 2, sizeof(double));
  p->work = (double *)calloc(2 * L2C_M, sizeof(double));
  p->wk = (double **)calloc(L, sizeof(double *));
  p->ck = (double **)calloc(L, sizeof(double *));
  p->wk[0] = (double *)calloc(Nb * 2 * L2C_M, sizeof(double));
  p->ck[0] = (double *)calloc(Nb * 2 * L2C_M, sizeof(double));
  for (size_t level = 1; level < L; level++) {
    const size_t b = get_number_of_blocks(level - 1);
    p->wk[level] = p->wk[level - 1] + b * 2 * L2C_M;
    p->ck[level] = p->ck[level - 1] + b * 2 * L2C_M;
  }
  return p;
}

void free_fmm(fmm_plan *p) {
  if (!p) return;
  if (p->gpu) l2c_gpu_plan_destroy((l2c_gpu_plan *)p->gpu);
  if (p->A) free(p->A);
  free(p->T);
  if (p->lagrange == 1) free(p->B); /* modal B points at the constant binomial table */
  free(p->ia);
  free(p->oa);
  free(p->work);
  if (p->wk) {
    free(p->wk[0]);
    free(p->wk);
  }
  if (p->ck) {
    free(p->ck[0]);
    free(p->ck);
  }
  if (p->dplan) free_direct(p->dplan);
  free(p);
}

size_t execute(const double *input_array, double *output_array, fmm_plan *fmmplan,
               size_t direction, const size_t stride) {
  host_err[0] = 0;
  if (!fmmplan || !fmmplan->gpu) {
    herr("null plan");
    return 0;
  }
  return l2c_gpu_execute((l2c_gpu_plan *)fmmplan->gpu, input_array, output_array, direction, 1,
                         0, stride, 0);
}

size_t execute_batched(const double *input_array, double *output_array, fmm_plan *fmmplan,
                       size_t direction, size_t count, size_t dist, size_t stride) {
  host_err[0] = 0;
  if (!fmmplan || !fmmplan->gpu) {
    herr("null plan");
    return 0;
  }
  return l2c_gpu_execute((l2c_gpu_plan *)fmmplan->gpu, input_array, output_array, direction,
                         count, dist, stride, 0);
}

/* Flop counts of directM / directL, leg2cheb.c:236-535. */
static size_t near_flops(const fmm_plan *p, size_t dir) {
  const size_t N = p->N, s = p->s, h = 2 * s, nL = N / h, i0 = (nL - 1) * h;
  size_t band = 0, f = 0;
  for (size_t n = (dir == 0 ? 0 : 2); n < 4 * s; n += 2) band += 3 * (n < h ? h : 2 * h - n);
  f += (nL - 1) * band;
  if (dir == 0) {
    for (size_t n = 0; 2 * n + i0 < N; n++) f += 3 * (N - (2 * n + i0));
    return f + N;
  }
  f += 3 * N;
  for (size_t n = 1; n < N - i0; n++) f += (N - (2 * n + i0)) * 3;
  return f + 2 * N;
}

size_t directM(const double *input_array, double *output_array, fmm_plan *fmmplan,
               const size_t strides) {
  host_err[0] = 0;
  if (!fmmplan || !fmmplan->gpu || fmmplan->L == 0) {
    herr("directM needs an FMM plan with L >= 1");
    return 0;
  }
  if (!l2c_gpu_execute((l2c_gpu_plan *)fmmplan->gpu, input_array, output_array, L2C, 1, 0,
                       strides, L2C_EXEC_NEAR_ONLY))
    return 0;
  return near_flops(fmmplan, 0);
}

size_t directL(const double *input, double *output_array, fmm_plan *fmmplan, size_t strides) {
  host_err[0] = 0;
  if (!fmmplan || !fmmplan->gpu || fmmplan->L == 0) {
    herr("directL needs an FMM plan with L >= 1");
    return 0;
  }
  if (!l2c_gpu_execute((l2c_gpu_plan *)fmmplan->gpu, input, output_array, C2L, 1, 0, strides,
                       L2C_EXEC_NEAR_ONLY))
    return 0;
  return near_flops(fmmplan, 1);
}

/* ------------------------------------------------------------------------ */
/* 2D, leg2cheb.c:1236-1297: all lines of an axis in one batched call.       */
/* ------------------------------------------------------------------------ */
fmm_plan_2d *create_fmm_2d(size_t N0, size_t N1, int axis, size_t maxs, size_t M,
                           size_t direction, const size_t lagrange, const size_t precompute,
                           size_t v) {
  fmm_plan_2d *p = (fmm_plan_2d *)calloc(1, sizeof(fmm_plan_2d));
  if (!p) return NULL;
  if (v > 1) printf("crate_fmm_2d\n");
  if (axis == 0) {
    p->fmmplan0 = create_fmm(N0, maxs, M, direction, lagrange, precompute, v);
  } else if (axis == 1) {
    p->fmmplan1 = create_fmm(N1, maxs, M, direction, lagrange, precompute, v);
  } else if (axis == -1) {
    p->fmmplan0 = create_fmm(N0, maxs, M, direction, lagrange, precompute, v);
    p->fmmplan1 = (N0 == N1) ? p->fmmplan0
                             : create_fmm(N1, maxs, M, direction, lagrange, precompute, v);
  }
  p->N0 = N0;
  p->N1 = N1;
  p->axis = axis;
  return p;
}

void free_fmm_2d(fmm_plan_2d *p) {
  if (!p) return;
  if (p->fmmplan0 == p->fmmplan1) {
    free_fmm(p->fmmplan0);
  } else {
    free_fmm(p->fmmplan0);
    free_fmm(p->fmmplan1);
  }
  free(p);
}

size_t execute2D(const double *input_array, double *output_array, fmm_plan_2d *p,
                 size_t direction) {
  host_err[0] = 0;
  if (!p) {
    herr("null plan");
    return 0;
  }
  const size_t N0 = p->N0, N1 = p->N1;
  if (p->axis == 0)
    return execute_batched(input_array, output_array, p->fmmplan0, direction, N1, 1, N1);
  if (p->axis == 1)
    return execute_batched(input_array, output_array, p->fmmplan1, direction, N0, N1, 1);
  if (p->axis == -1) {
    double *tmp = (double *)calloc(N0 * N1, sizeof(double));
    if (!tmp) {
      herr("out of host memory");
      return 0;
    }
    size_t f = execute_batched(input_array, tmp, p->fmmplan0, direction, N1, 1, N1);
    if (f) {
      const size_t f1 = execute_batched(tmp, output_array, p->fmmplan1, direction, N0, N1, 1);
      f = f1 ? f + f1 : 0;
    }
    free(tmp);
    return f;
  }
  herr("axis must be 0, 1 or -1");
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Ragged batches (extension)                                                */
/* ------------------------------------------------------------------------ */
fmm_plan_ragged *create_fmm_ragged(size_t count, const size_t *N, size_t maxs, size_t M,
                                   size_t direction, size_t lagrange, size_t precompute,
                                   size_t v) {
  host_err[0] = 0;
  if (M != L2C_M || lagrange != 0) {
    herr("only the modal form with M = 18 is implemented");
    return NULL;
  }
  fmm_plan_ragged *p = (fmm_plan_ragged *)calloc(1, sizeof(fmm_plan_ragged));
  if (!p) {
    herr("out of host memory");
    return NULL;
  }
  l2c_gpu_ragged *g =
      l2c_gpu_ragged_create(count, N, maxs, direction, precompute ? L2C_PLAN_PRECOMPUTE_NEAR : 0);
  if (!g) {
    free(p);
    return NULL;
  }
  p->count = count;
  p->total = l2c_gpu_ragged_total(g);
  p->maxs = maxs;
  p->direction = direction;
  p->gpu = g;
  if (v > 1) printf("ragged plan: %zu vectors, %zu coefficients\n", count, p->total);
  return p;
}

size_t execute_ragged(const double *input_array, double *output_array, fmm_plan_ragged *p,
                      size_t direction) {
  host_err[0] = 0;
  if (!p || !p->gpu) {
    herr("null plan");
    return 0;
  }
  return l2c_gpu_ragged_execute((l2c_gpu_ragged *)p->gpu, input_array, output_array, direction,
                                0);
}

void free_fmm_ragged(fmm_plan_ragged *p) {
  if (!p) return;
  if (p->gpu) l2c_gpu_ragged_destroy((l2c_gpu_ragged *)p->gpu);
  free(p);
}
