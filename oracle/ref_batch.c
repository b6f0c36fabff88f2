/* TEST INFRASTRUCTURE -- CPU baseline harness around the UNMODIFIED reference.
 *
 * Loops the reference's execute() (src/C/leg2cheb.c:1299-1500, compiled from the
 * reference's own sources into libleg2cheb_ref.so by oracle/Makefile) over a
 * batch of vectors, the way a caller of the reference transforms many vectors:
 * plans are not reentrant (their scratch ia/oa/wk/ck lives in the plan,
 * leg2cheb.c:1195-1211), so every OpenMP thread owns its own plans, one per
 * distinct length among the vectors it is given.  Vectors are dealt to threads
 * longest first, each to the thread with the least work so far (work ~ N).
 * Inside a thread the reference runs serially: nested OpenMP regions are
 * inactive and OpenBLAS is set to one thread while a batch runs.
 *
 * Used only by bench.py (the reference arm and the CPU baseline) and tests/.
 * Planning happens in ref_batch_create, outside any timed region. */
#define _GNU_SOURCE /* qsort_r */
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "cblas.h"
#include "leg2cheb.h"

typedef struct {
  size_t nvec;     /* vectors of this thread */
  size_t *vec;     /* their indices */
  fmm_plan **plan; /* plan of each of them (shared between equal lengths) */
  fmm_plan **own;  /* distinct plans this thread created */
  size_t nown;
} thread_work;

typedef struct {
  size_t count, threads;
  size_t *N, *off;  /* lengths and offsets in the packed arrays */
  thread_work *tw;
} ref_batch;

static int by_length_desc(const void *a, const void *b, void *N_) {
  const size_t *N = (const size_t *)N_;
  const size_t x = *(const size_t *)a, y = *(const size_t *)b;
  return N[x] < N[y] ? 1 : N[x] > N[y] ? -1 : (x > y) - (x < y);
}

/* Threads of a single-vector call: the reference's OpenMP loops and OpenBLAS.
 * (Its step-3 dgemv calls run inside OpenMP loops, leg2cheb.c:1404-1435, so a
 * threaded OpenBLAS there oversubscribes the cores.) */
void ref_set_threads(int omp_threads, int blas_threads) {
  omp_set_num_threads(omp_threads);
  openblas_set_num_threads(blas_threads);
}

void ref_batch_free(ref_batch *b) {
  if (!b) return;
  for (size_t t = 0; t < b->threads; t++) {
    for (size_t i = 0; i < b->tw[t].nown; i++) free_fmm(b->tw[t].own[i]);
    free(b->tw[t].vec);
    free(b->tw[t].plan);
    free(b->tw[t].own);
  }
  free(b->tw);
  free(b->N);
  free(b->off);
  free(b);
}

/* count vectors of lengths N[0..count) packed back to back; maxs as create_fmm;
 * threads: OpenMP threads (each with its own plans). */
ref_batch *ref_batch_create(size_t count, const size_t *N, size_t maxs, size_t threads) {
  if (count == 0 || threads == 0) return NULL;
  ref_batch *b = calloc(1, sizeof(*b));
  b->count = count;
  b->threads = threads;
  b->N = malloc(count * sizeof(size_t));
  b->off = malloc((count + 1) * sizeof(size_t));
  memcpy(b->N, N, count * sizeof(size_t));
  b->off[0] = 0;
  for (size_t v = 0; v < count; v++) b->off[v + 1] = b->off[v] + N[v];
  b->tw = calloc(threads, sizeof(thread_work));
  size_t *order = malloc(count * sizeof(size_t));
  for (size_t v = 0; v < count; v++) order[v] = v;
  qsort_r(order, count, sizeof(size_t), by_length_desc, b->N);
  size_t *load = calloc(threads, sizeof(size_t));
  for (size_t t = 0; t < threads; t++) {
    b->tw[t].vec = malloc(count * sizeof(size_t));
    b->tw[t].plan = malloc(count * sizeof(fmm_plan *));
    b->tw[t].own = malloc(count * sizeof(fmm_plan *));
  }
  for (size_t i = 0; i < count; i++) {
    size_t best = 0;
    for (size_t t = 1; t < threads; t++)
      if (load[t] < load[best]) best = t;
    thread_work *w = &b->tw[best];
    w->vec[w->nvec++] = order[i];
    load[best] += N[order[i]];
  }
  free(order);
  free(load);
  int ok = 1;
  /* each thread plans for its own vectors (vectors arrive longest first, so
   * equal lengths are adjacent) */
#pragma omp parallel num_threads((int)threads) reduction(&& : ok)
  {
    const int t = omp_get_thread_num();
    thread_work *w = &b->tw[t];
    for (size_t i = 0; i < w->nvec; i++) {
      const size_t n = N[w->vec[i]];
      if (i > 0 && N[w->vec[i - 1]] == n) {
        w->plan[i] = w->plan[i - 1];
        continue;
      }
      fmm_plan *p = create_fmm(n, maxs, 18, 2, 0, 0, 0);
      if (!p) ok = 0;
      w->own[w->nown++] = p;
      w->plan[i] = p;
    }
  }
  if (!ok) {
    ref_batch_free(b);
    return NULL;
  }
  return b;
}

/* out += transform(in) for every vector (the caller zeroes out, as every caller
 * of the reference does); returns the summed flop count. */
size_t ref_batch_execute(ref_batch *b, const double *in, double *out, size_t direction) {
  size_t flops = 0;
  const int levels = omp_get_max_active_levels();
  omp_set_max_active_levels(1);
  openblas_set_num_threads(1);
#pragma omp parallel num_threads((int)b->threads) reduction(+ : flops)
  {
    thread_work *w = &b->tw[omp_get_thread_num()];
    for (size_t i = 0; i < w->nvec; i++) {
      const size_t v = w->vec[i];
      flops += execute(in + b->off[v], out + b->off[v], w->plan[i], direction, 1);
    }
  }
  omp_set_max_active_levels(levels);
  return flops;
}
