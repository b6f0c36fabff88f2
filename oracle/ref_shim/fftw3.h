/* Minimal stand-in for <fftw3.h>, used ONLY to compile the unmodified reference
 * sources (src/C/leg2cheb.c, lambda.c, dct.c, src/bin/l2c.c) into the test
 * oracle under oracle/_ref.  FFTW itself is not installed in this image.
 *
 * On the reference's default path (M = 18, lagrange = 0, leg2cheb.c:893) FFTW is
 * only used for fftw_malloc/fftw_free, which map to posix_memalign/free here.
 * Every planner/executor entry point aborts, so a code path that would really
 * need FFTW fails loudly instead of producing wrong numbers. */
#ifndef L2C_ORACLE_FFTW3_SHIM_H
#define L2C_ORACLE_FFTW3_SHIM_H
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double _Complex fftw_complex;
typedef struct l2c_shim_fftw_plan_s *fftw_plan;
typedef int fftw_r2r_kind;
enum { FFTW_REDFT10 = 5 };
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_r2r_1d(int n, double *in, double *out, fftw_r2r_kind kind, unsigned flags);
fftw_plan fftw_plan_r2r_2d(int n0, int n1, double *in, double *out, fftw_r2r_kind k0,
                           fftw_r2r_kind k1, unsigned flags);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void fftw_flops(const fftw_plan p, double *add, double *mul, double *fma);
void fftw_print_plan(const fftw_plan p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int n);
void fftw_cleanup(void);
void fftw_cleanup_threads(void);
int fftw_import_wisdom_from_filename(const char *f);
int fftw_export_wisdom_to_filename(const char *f);
#ifdef __cplusplus
}
#endif
#endif
