/* l2c_cuda.h -- thin C ABI between the host C library (libleg2cheb.so) and the
 * sm_103a CUDA implementation (libl2c_cuda.so).  Plain pointers and sizes only.
 *
 * Each entry point replaces a piece of the reference's src/C/leg2cheb.c:
 *   l2c_gpu_plan_create   <- create_fmm / create_direct   (leg2cheb.c:820-1234, 758-818)
 *   l2c_gpu_execute       <- execute / direct             (leg2cheb.c:1299-1500, 152-234)
 *   l2c_gpu_near          <- directM / directL            (leg2cheb.c:236-376, 378-535)
 *   l2c_gpu_plan_destroy  <- free_fmm / free_direct       (leg2cheb.c:688-756, 650-673)
 *   l2c_lambda            <- Lambda                       (lambda.c:65-98)
 *   l2c_lambda_int        <- LambdaI                      (lambda.c:101-191)
 * Errors never abort: calls return 0 / NULL and l2c_gpu_last_error() explains.
 */
#ifndef L2C_CUDA_H
#define L2C_CUDA_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct l2c_gpu_plan l2c_gpu_plan;

/* Plan flags */
#define L2C_PLAN_DIRECT_ONLY 1u     /* O(N^2) direct sums whatever N (create_direct)  */
#define L2C_PLAN_PRECOMPUTE_NEAR 2u /* keep the near-field band weights in device memory
                                       (3s^2+s doubles per 2s coefficients and direction;
                                       the reference's `precompute`, leg2cheb.c:1108-1193):
                                       one FP64 FMA per band term instead of two ops */

#define L2C_PLAN_MIXED 4u /* mixed form: leaf, transfer and far-field products on
                                FP16 tensor cores, FP64-accurate (operands split into
                                exact 9-bit digit slices, products recombined exactly
                                in integers; no FP64 instructions); for batches at
                                s = 16 or 32 also the full blocks of the near-field band;
                                the rest of the band, accumulation and scaling in FP64.
                                Leaf sizes s <= 64. */

#define L2C_PLAN_NODAL 8u /* nodal (Lagrange) form, create_fmm's lagrange = 1
                                (leg2cheb.c:997-1031, 1076-1100): leaf matrices of
                                barycentric interpolation weights, far-field blocks
                                of kernel samples, transfer matrices B0 | B1.
                                Not combinable with L2C_PLAN_MIXED. */

/* Execute flags */
#define L2C_EXEC_ASYNC 1u       /* return without waiting (device pointers only)  */
#define L2C_EXEC_NEAR_ONLY 2u   /* near-field band + final scaling only (directM/L) */

/* Geometry of create_fmm (leg2cheb.c:860-871): L = ceil(log2(N/maxs)) - 2,
 * s = ceil(N / 2^(L+2)), Nn = s 2^(L+2); L = 0 selects the direct method.
 * Returns L. */
size_t l2c_geometry(size_t N, size_t maxs, size_t *s, size_t *Nn);

/* Build the device plan: Lambda tables, the leaf matrices T, the far-field
 * blocks A for each planned direction (directions: 0 L2C, 1 C2L, 2 both), all on
 * the current CUDA device.  M = 18; modal form unless L2C_PLAN_NODAL. */
l2c_gpu_plan *l2c_gpu_plan_create(size_t N, size_t maxs, size_t directions, unsigned flags);
void l2c_gpu_plan_destroy(l2c_gpu_plan *plan);

/* info[0..7] = N, L, s, Nn, number of blocks N_b, M, planned directions, maxs */
int l2c_gpu_plan_info(const l2c_gpu_plan *plan, size_t *info);

/* count transforms of length N: vector v reads in[v*dist + i*stride] and
 * updates out[v*dist + i*stride], i < N, with the reference's contract
 * (FMM: out = scale (out + far + near); direct: out overwritten).  in/out may be
 * host or device pointers.  Returns the reference's flop count times count,
 * 0 on failure. */
size_t l2c_gpu_execute(l2c_gpu_plan *plan, const double *in, double *out, size_t direction,
                       size_t count, size_t dist, size_t stride, unsigned flags);

/* Wait for work queued with L2C_EXEC_ASYNC.  0 on success. */
int l2c_gpu_synchronize(l2c_gpu_plan *plan);

/* The plan's CUDA stream (a cudaStream_t), for callers timing device work. */
void *l2c_gpu_plan_stream(l2c_gpu_plan *plan);

/* Reference flop count of one transform in this direction (0 if unplanned). */
size_t l2c_gpu_flops(const l2c_gpu_plan *plan, size_t direction);

/* Kernel launches this plan has issued since it was created. */
size_t l2c_gpu_launch_count(const l2c_gpu_plan *plan);

/* Per-phase accounting.  Phases, in launch order: */
#define L2C_PHASE_GATHER 0    /* strided / premultiplied input copy        */
#define L2C_PHASE_NEAR 1      /* near-field band                           */
#define L2C_PHASE_LEAF_UP 2   /* leaf values -> Chebyshev coefficients     */
#define L2C_PHASE_TREE_UP 3   /* upward transfer, all levels               */
#define L2C_PHASE_FAR 4       /* far-field blocks, all levels              */
#define L2C_PHASE_TREE_DOWN 5 /* downward transfer, all levels             */
#define L2C_PHASE_LEAF_DOWN 6 /* back to leaf values + scaling             */
#define L2C_PHASE_DIRECT 7    /* O(N^2) direct method (L < 1)              */
#define L2C_NPHASES 8
/* Enable (1) or disable (0) CUDA-event timing of each phase on the plan's
 * stream, and reset the counters.  0 on success. */
int l2c_gpu_profile(l2c_gpu_plan *plan, int enable);
/* Accumulated milliseconds and launches per phase since the last reset
 * (arrays of L2C_NPHASES; either may be NULL).  Waits for recorded events.
 * Returns L2C_NPHASES. */
int l2c_gpu_profile_read(l2c_gpu_plan *plan, double *ms, size_t *launches);

/* Autotuner (no reference counterpart: the reference runs one code path on
 * the CPU).  For one call shape -- direction, count, dist, stride, as passed to
 * l2c_gpu_execute -- it times this plan's launch choices on synthetic device
 * data and keeps the fastest for every later call of that shape: the band on a
 * second stream or not and the chain step after which it starts, programmatic
 * dependent launch, the chain's priority, the band's CTA size, vectors per
 * thread and grid cap, the mixed form's tile buffers, and whether the band
 * reads its weights from a table in device memory (by default: batches whose
 * table is no larger than their input).  No choice changes results: outputs
 * are the same bits under every setting.  Blocks while it runs (tens of calls
 * of the shape).
 * Returns the tuned milliseconds per call, 0 on error (l2c_gpu_last_error).
 * With L2C_AUTOTUNE=1 in the environment at plan creation, each new shape is
 * tuned on its first call; with L2C_AUTOTUNE_CACHE=path, tuned shapes are
 * appended to that file and plans of the same device, N, maxs and form read
 * them back instead of tuning again. */
double l2c_gpu_autotune(l2c_gpu_plan *plan, size_t direction, size_t count, size_t dist,
                        size_t stride);
/* The launch choices a call shape runs with, as text into buf ("overlap=1
 * pdl=1 ..."); ms (may be NULL) receives the tuned and the default
 * milliseconds per call when tuned.  Returns 1 if the shape was tuned by this
 * plan, 2 if its choices came from the cache file, 0 if the plan's own choices
 * apply, -1 for a null plan. */
int l2c_gpu_tuned_config(l2c_gpu_plan *plan, size_t direction, size_t count, size_t dist,
                         size_t stride, char *buf, size_t len, double *ms);

/* Copy plan tables to host memory, for checking plan construction.
 * which: 0 = A[L2C], 1 = A[C2L], 2 = Lambda table a, 3 = an, 4 = dn, 5 = T,
 * 6 = nodal transfer matrices B0 | B1 (2 M^2; nodal plans only).
 * Returns the number of doubles copied (n_max caps it), 0 if absent. */
size_t l2c_gpu_plan_copy(const l2c_gpu_plan *plan, int which, double *dst, size_t n_max);

/* One transform that allocates no device memory (no counterpart in the
 * reference).  For callers that cannot allocate at transform time -- an
 * application that reserves the device for its own memory pool, a solver that
 * must not risk allocation latency or failure inside a time step.  It runs the
 * plain FP64 kernels of l2c_gpu_execute (count = 1), but the working buffers
 * live in a fixed array of L2C_NOALLOC_SCRATCH_DOUBLES doubles (4 MiB) that
 * every GPU loading this library holds until the process exits; the plan's own
 * tables are built beforehand by l2c_gpu_plan_create, as set-up.
 *   - in and out must be device pointers; FMM plans only (L >= 1).
 *   - a plan needing more than the fixed array (2N + 144 N_b doubles; e.g.
 *     N up to about 1.2e5 at maxs = 64) is rejected with an error message.
 *   - plain and nodal plans give the same results as l2c_gpu_execute.  On a
 *     plan made with L2C_PLAN_MIXED it still runs the FP64 far field (such a
 *     plan keeps the FP64 blocks; its tensor-core fragments are built on the
 *     first batched call, which allocates), so the results agree with
 *     l2c_gpu_execute within 1e-14 but not bit for bit, and a vector holding
 *     an Inf or NaN gets the plain form's pattern of non-finite outputs.
 *   - the first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress), so make that first call before any stream capture.
 *   - calls on one device are serialised, since all of them share the array:
 *     each call waits on the host until its work has finished on the GPU (it
 *     synchronises the plan's stream) before it returns.
 * Returns the reference's flop count, 0 on failure (l2c_gpu_last_error()). */
#define L2C_NOALLOC_SCRATCH_DOUBLES (1u << 19)
size_t l2c_gpu_execute_noalloc(l2c_gpu_plan *plan, const double *in, double *out,
                               size_t direction, size_t stride);

/* Ragged batches: count vectors of lengths N[0..count) (packed back to back in
 * the caller's arrays: vector v starts at N[0] + ... + N[v-1]), each transformed
 * exactly as execute() with create_fmm(N[v], maxs, 18, directions, 0, 0, 0)
 * would (vectors with L < 1 take the direct method), in one set of launches whose
 * count does not depend on the number of vectors.  flags: L2C_PLAN_PRECOMPUTE_NEAR
 * keeps the band weights of each leaf size in the list in device memory (one
 * table per leaf size, serving every vector with it; the same bits, one FP64
 * instruction per band term instead of two).  No counterpart in the reference
 * (its callers loop execute over plans, src/bin/l2c.c harnesses). */
typedef struct l2c_gpu_ragged l2c_gpu_ragged;
l2c_gpu_ragged *l2c_gpu_ragged_create(size_t count, const size_t *N, size_t maxs,
                                      size_t directions, unsigned flags);
void l2c_gpu_ragged_destroy(l2c_gpu_ragged *plan);
/* host or device pointers; returns the summed reference flop count, 0 on failure */
size_t l2c_gpu_ragged_execute(l2c_gpu_ragged *plan, const double *in, double *out,
                              size_t direction, unsigned flags);
int l2c_gpu_ragged_synchronize(l2c_gpu_ragged *plan);
size_t l2c_gpu_ragged_total(const l2c_gpu_ragged *plan);            /* sum of N */
size_t l2c_gpu_ragged_flops(const l2c_gpu_ragged *plan, size_t direction);
void *l2c_gpu_ragged_stream(l2c_gpu_ragged *plan);
size_t l2c_gpu_ragged_launch_count(const l2c_gpu_ragged *plan);
/* Autotuner of a ragged list, per direction: the band (and the direct-method
 * vectors) on a second stream beside the far-field chain or not, and the
 * chain's kernels at the device's greatest priority or not, timed on synthetic
 * data of the list (the same bits under every choice).  Returns the tuned ms
 * per call, 0 on error.  L2C_AUTOTUNE=1 at creation tunes on each direction's
 * first call; L2C_OVERLAP / L2C_CHAIN_PRIO set the untuned choices. */
double l2c_gpu_ragged_autotune(l2c_gpu_ragged *plan, size_t direction);
/* "overlap=.. prio=.." into buf; ms (may be NULL) gets the tuned and default
 * ms per call.  Returns 1 if tuned, 0 if the plan's own choices apply, -1 on a
 * bad argument. */
int l2c_gpu_ragged_tuned_config(l2c_gpu_ragged *plan, size_t direction, char *buf, size_t len,
                                double *ms);

/* Lambda(z) and Lambda at integer z, host side, bit-identical to the device. */
double l2c_lambda(double z);
double l2c_lambda_int(size_t z);

/* Last error message of the calling thread ("" if none). */
const char *l2c_gpu_last_error(void);

/* Library version string. */
const char *l2c_gpu_version(void);

#ifdef __cplusplus
}
#endif
#endif
