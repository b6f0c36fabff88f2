/* leg2cheb.h -- drop-in public API of the GB300 Legendre<->Chebyshev transform.
 *
 * Same enum, structs and prototypes as the reference's src/C/leg2cheb.h
 * (spectralDNS/Legendre-to-Chebyshev), so the reference's ctypes wrapper
 * (src/ctypes/l2ctypes.py), Cython module (src/cython/l2c.pyx) and `l2c` driver
 * (src/bin/l2c.c) compile and link against libleg2cheb.so unchanged.
 *
 * Differences a caller can see (all extensions, none removes behaviour):
 *  - fmm_plan and direct_plan carry one extra trailing field, `gpu`, the
 *    device-side plan.  Fields before it keep the reference's order and types.
 *  - execute() returns the reference's flop count on success and 0 on failure
 *    (unplanned direction, CUDA error); l2c_last_error() says why.  The
 *    reference asserts or dereferences NULL in those cases.
 *  - in/out may be host pointers or device pointers (used in place).  Pageable
 *    host memory is copied to and from the GPU; page-locked host memory is read
 *    and written in place by the kernels through its device mapping.
 */
#ifndef LEG2CHEB_H
#define LEG2CHEB_H

#include <assert.h>
#include <errno.h>
#include <math.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#if !defined(_WIN32)
#include <sys/resource.h>
#include <unistd.h>
#endif

/* The reference header pulls in FFTW and CBLAS, and its `l2c` driver relies on
 * that for its own FFTW/BLAS test modes.  The library itself needs neither. */
#if defined(__has_include)
#if __has_include(<complex.h>) && !defined(__cplusplus)
#include <complex.h>
#endif
#if __has_include(<fftw3.h>)
#include <fftw3.h>
#define L2C_HAVE_FFTW_TYPES 1
#endif
#if __has_include(<cblas.h>)
#include <cblas.h>
#endif
#endif
#if defined(OMP)
#include <omp.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* leg2cheb.h:27 */
enum { L2C = 0, C2L = 1, BOTH = 2 };

/* Wall-clock helpers used by the `l2c` driver, leg2cheb.h:29-46 (CLOCK_MONOTONIC). */
#ifndef tic
#define tic                                                                    \
  ({                                                                           \
    struct timespec l2c_ts_;                                                   \
    clock_gettime(CLOCK_MONOTONIC, &l2c_ts_);                                  \
    (uint64_t)(l2c_ts_.tv_sec * 1e9 + l2c_ts_.tv_nsec);                        \
  })
#define toc(start)                                                             \
  ({                                                                           \
    struct timespec l2c_ts_;                                                   \
    clock_gettime(CLOCK_MONOTONIC, &l2c_ts_);                                  \
    uint64_t l2c_end_ = (uint64_t)(l2c_ts_.tv_sec * 1.0E9 + l2c_ts_.tv_nsec); \
    (l2c_end_ - (start)) * 1.0E-9;                                             \
  })
#define dtics(a, b) (double)(b - a) * 1.0E-9
#endif

/* leg2cheb.h:48-56.  Host copies of the Lambda tables; gpu is the device plan. */
typedef struct {
  size_t direction;
  size_t N;
  double *a;
  double *dn;
  double *an;
  double *lf;
  double *lb;
  void *gpu;
} direct_plan;

/* leg2cheb.h:58-78.  Host-side fields keep the reference's meaning: T, B, BT,
 * and the per-level views wk/ck/ia/oa/work are host buffers of the same sizes
 * (the `l2c` driver's matvectri and dgemm probes read them); A[dir] is NULL on
 * the host -- the far-field blocks are assembled and kept on the GPU only. */
typedef struct {
  size_t direction;
  size_t M;
  size_t N;
  size_t Nn;
  size_t L;
  size_t s;
  size_t lagrange;
  double **A;
  double *T;
  double *B;
  double *BT;
  double *ia;
  double *oa;
  double *work;
  double **wk;
  double **ck;
  double **lf;
  double **lb;
  direct_plan *dplan;
  void *gpu;
} fmm_plan;

/* leg2cheb.h:80-86 */
typedef struct {
  fmm_plan *fmmplan0;
  fmm_plan *fmmplan1;
  size_t N0;
  size_t N1;
  int axis;
} fmm_plan_2d;

/* leg2cheb.h:88-129 */
void free_fmm(fmm_plan *plan);
void free_fmm_2d(fmm_plan_2d *plan);
void free_direct(direct_plan *dplan);
fmm_plan_2d *create_fmm_2d(size_t N0, size_t N1, int axis, size_t maxs, size_t M,
                           size_t direction, const size_t lagrange, const size_t precompute,
                           size_t v);
fmm_plan *create_fmm(const size_t N, const size_t maxs, const size_t M, const size_t direction,
                     const size_t lagrange, const size_t precompute, const size_t v);
direct_plan *create_direct(size_t N, size_t direction, const size_t precompute);
size_t direct(const double *input_array, double *output_array, direct_plan *dplan,
              size_t direction, size_t stride);
size_t directM(const double *input_array, double *output_array, fmm_plan *fmmplan,
               const size_t strides);
size_t directL(const double *input, double *output_array, fmm_plan *fmmplan, size_t strides);
size_t execute2D(const double *input_array, double *output_array, fmm_plan_2d *fmmplan2d,
                 size_t direction);
size_t execute(const double *input_array, double *output_array, fmm_plan *fmmplan,
               size_t direction, const size_t stride);
void matvectri(const double *A, const double *x, double *b, const size_t m, const bool upper);
size_t get_number_of_blocks(const size_t level);
size_t get_total_number_of_blocks(const size_t L);
size_t get_h(const size_t level, const size_t L);
size_t get_number_of_submatrices(const size_t level);
size_t get_total_number_of_submatrices(const size_t L);
void get_ij(size_t *ij, const size_t level, const size_t block, const size_t s, const size_t L);

double _Lambda0(const double z);
double _LambdaE(const double z);
double Lambda(const double z);
double LambdaI(const size_t z);
void Lambdavec(const double *z, double *w, const size_t N);

/* 18-point DCT-II helpers of the reference (src/C/dct.c).  Same results; the
 * complex argument of fft9/fft9c is an array of {re, im} pairs. */
void dct2(double *input, double *output);
void dct(double *input, double *output, size_t st);
void dct0(double *input, double *output, size_t st);
void dct_radix2(double *input, double *output, size_t st);
void dct_radix23(double *input, double *output, size_t st);
void dct_fft(double *input, double *output, size_t st);
#if defined(L2C_HAVE_FFTW_TYPES)
void fft9c(fftw_complex *x);
void fft9(fftw_complex *x);
#else
void fft9c(double (*x)[2]);
void fft9(double (*x)[2]);
#endif

/* Extensions (no counterpart in the reference) */

/* Reason for the last failure on this thread ("" when none). */
const char *l2c_last_error(void);

/* Many transforms with one plan in one call: vector v reads
 * input_array[v*dist + i*stride] and writes output_array[v*dist + i*stride],
 * i < N.  Same per-vector semantics as execute().  Returns the summed flop
 * count, 0 on failure. */
size_t execute_batched(const double *input_array, double *output_array, fmm_plan *fmmplan,
                       size_t direction, size_t count, size_t dist, size_t stride);

/* create_fmm with extra plan options (bit flags):
 *   L2C_FMM_MIXED   the mixed form: leaf, transfer and far-field products on FP16
 *                   tensor cores, FP64-accurate (exact 9-bit digit slices, exact
 *                   integer recombination), for batches at leaf size 16 or 32 also
 *                   the full blocks of the near-field band; the rest of the band,
 *                   accumulation and scaling in FP64 (maxs <= 64)
 * Same semantics as create_fmm otherwise. */
#define L2C_FMM_MIXED 1u
fmm_plan *create_fmm_ex(const size_t N, const size_t maxs, const size_t M, const size_t direction,
                        const size_t lagrange, const size_t precompute, const size_t v,
                        unsigned flags);

/* Ragged batch: count vectors of lengths N[0..count), packed back to back
 * (vector v starts at N[0] + ... + N[v-1]); each is transformed exactly as
 * execute() with create_fmm(N[v], maxs, M, direction, ...) would, all in one set
 * of GPU launches; precompute = 1 keeps the band weights in device memory, as
 * create_fmm's does (one table per leaf size in the list).  Returns the summed
 * flop count, 0 on failure. */
typedef struct {
  size_t count;
  size_t total; /* sum of N */
  size_t maxs;
  size_t direction;
  void *gpu;
} fmm_plan_ragged;
fmm_plan_ragged *create_fmm_ragged(size_t count, const size_t *N, size_t maxs, size_t M,
                                   size_t direction, size_t lagrange, size_t precompute, size_t v);
size_t execute_ragged(const double *input_array, double *output_array, fmm_plan_ragged *plan,
                      size_t direction);
void free_fmm_ragged(fmm_plan_ragged *plan);

#ifdef __cplusplus
}
#endif
#endif
