/* Minimal stand-in for <cblas.h>, used ONLY to compile the unmodified reference
 * sources into the test oracle under oracle/_ref.  The two BLAS routines the
 * reference calls (cblas_dgemm at leg2cheb.c:1381,1467 and cblas_dgemv at
 * leg2cheb.c:1409-1432,1457-1460) are routed to the OpenBLAS build that scipy
 * bundles (32-bit integer interface, symbols prefixed with "scipy_"). */
#ifndef L2C_ORACLE_CBLAS_SHIM_H
#define L2C_ORACLE_CBLAS_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
void scipy_cblas_dgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE, int, int,
                       int, double, const double *, int, const double *, int, double, double *,
                       int);
void scipy_cblas_dgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, int, int, double, const double *,
                       int, const double *, int, double, double *, int);
void scipy_openblas_set_num_threads(int);
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dgemv scipy_cblas_dgemv
#define openblas_set_num_threads scipy_openblas_set_num_threads
#ifdef __cplusplus
}
#endif
#endif
