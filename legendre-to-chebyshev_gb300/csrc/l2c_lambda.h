/* Lambda(z) = Gamma(z+1/2)/Gamma(z+1), shared by the host library and the GPU
 * kernels so both produce bit-identical tables.
 *
 * Algorithm (the one the reference uses, lambda.c:65-98 and 101-191):
 *   - integer z < 256: correctly rounded table (l2c_tables.h);
 *   - z >= 10: Lambda(z) = (1/sqrt(z+1/4)) * sum_k c_k w^k, w = (z+1/4)^-2, with
 *     c_k from l2c_tables.h; the series is cut after 1, 2, 3, 4, 5, 6 or 7 terms
 *     for z > 2014, > 141, > 40, > 20, > 14, or below (the reference's cut
 *     points, which keep the truncation error below half an ulp);
 *   - z < 10: Lambda(z) = Lambda(z+1) (z+1)/(z+1/2), applied upward.
 * Every operation is an explicitly rounded IEEE operation (no contraction),
 * so host (-ffp-contract=off) and device agree to the bit. */
#ifndef L2C_LAMBDA_H
#define L2C_LAMBDA_H

#include <stddef.h>

#include "l2c_tables.h"

#if defined(__CUDACC__)
#define L2C_HD __host__ __device__ __forceinline__
#else
#define L2C_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define L2C_ADD(a, b) __dadd_rn((a), (b))
#define L2C_SUB(a, b) __dsub_rn((a), (b))
#define L2C_MUL(a, b) __dmul_rn((a), (b))
#define L2C_DIV(a, b) __ddiv_rn((a), (b))
#define L2C_SQRT(a) __dsqrt_rn((a))
#else
#include <math.h>
#define L2C_ADD(a, b) ((a) + (b))
#define L2C_SUB(a, b) ((a) - (b))
#define L2C_MUL(a, b) ((a) * (b))
#define L2C_DIV(a, b) ((a) / (b))
#define L2C_SQRT(a) sqrt((a))
#endif

/* Series part, valid for z >= 10. */
L2C_HD double l2c_lambda_series(double z) {
  const double zp = L2C_ADD(z, 0.25);
  const double sc = L2C_DIV(1.0, L2C_SQRT(zp));
  const double w = L2C_DIV(1.0, L2C_MUL(zp, zp));
  double y = L2C_ADD(1.0, L2C_MUL(L2C_LAMBDA_C1, w));
  if (z > 2014) return L2C_MUL(y, sc);
  double wk = L2C_MUL(w, w);
  y = L2C_ADD(y, L2C_MUL(L2C_LAMBDA_C2, wk));
  if (z > 141) return L2C_MUL(y, sc);
  wk = L2C_MUL(wk, w);
  y = L2C_ADD(y, L2C_MUL(L2C_LAMBDA_C3, wk));
  if (z > 40) return L2C_MUL(y, sc);
  wk = L2C_MUL(wk, w);
  y = L2C_ADD(y, L2C_MUL(L2C_LAMBDA_C4, wk));
  if (z > 20) return L2C_MUL(y, sc);
  wk = L2C_MUL(wk, w);
  y = L2C_ADD(y, L2C_MUL(L2C_LAMBDA_C5, wk));
  if (z > 14) return L2C_MUL(y, sc);
  wk = L2C_MUL(wk, w);
  y = L2C_ADD(y, L2C_MUL(L2C_LAMBDA_C6, wk));
  return L2C_MUL(y, sc);
}

/* Lambda(z) for any z > -1/2.  Below 10 the argument is stepped up by ones
 * (each step rounded, as a recursive evaluation would), the series is taken
 * there, and the ratio (z+1)/(z+1/2) is applied back down. */
#define L2C_LAMBDA_MAX_STEPS 64
L2C_HD double l2c_lambda_eval(double z) {
  if (!(z < 10)) return l2c_lambda_series(z);
  double zs[L2C_LAMBDA_MAX_STEPS + 1];
  int n = 0;
  zs[0] = z;
  while (zs[n] < 10 && n < L2C_LAMBDA_MAX_STEPS) {
    zs[n + 1] = L2C_ADD(zs[n], 1.0);
    n++;
  }
  double v = l2c_lambda_series(zs[n]);
  for (int k = n - 1; k >= 0; k--)
    v = L2C_DIV(L2C_MUL(v, L2C_ADD(zs[k], 1.0)), L2C_ADD(zs[k], 0.5));
  return v;
}

#endif
