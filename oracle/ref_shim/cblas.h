/* Minimal stand-in for <cblas.h>, used ONLY to compile the unmodified reference
 * sources into the test oracle under oracle/_ref.  The two BLAS routines the
 * reference calls (cblas_dgemm at leg2cheb.c:1381,1467 and cblas_dgemv at
 * leg2cheb.c:1409-1432,1457-1460) are routed to an OpenBLAS build that a Python
 * package bundles:
 *   default               scipy's: 32-bit integers, symbols prefixed "scipy_"
 *   L2C_SHIM_OPENBLAS64   numpy's: 64-bit integers, symbols prefixed "scipy_" and
 *                         suffixed "64_" (the prototypes below take long long, so
 *                         the reference's int arguments are converted at the call) */
#ifndef L2C_ORACLE_CBLAS_SHIM_H
#define L2C_ORACLE_CBLAS_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
#ifdef L2C_SHIM_OPENBLAS64
typedef long long l2c_blasint;
#define L2C_BLAS(name) scipy_##name##64_
#else
typedef int l2c_blasint;
#define L2C_BLAS(name) scipy_##name
#endif
void L2C_BLAS(cblas_dgemm)(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE,
                           l2c_blasint, l2c_blasint, l2c_blasint, double, const double *,
                           l2c_blasint, const double *, l2c_blasint, double, double *,
                           l2c_blasint);
void L2C_BLAS(cblas_dgemv)(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, l2c_blasint, l2c_blasint,
                           double, const double *, l2c_blasint, const double *, l2c_blasint,
                           double, double *, l2c_blasint);
void L2C_BLAS(openblas_set_num_threads)(int);
#define cblas_dgemm L2C_BLAS(cblas_dgemm)
#define cblas_dgemv L2C_BLAS(cblas_dgemv)
#define openblas_set_num_threads L2C_BLAS(openblas_set_num_threads)
#ifdef __cplusplus
}
#endif
#endif
