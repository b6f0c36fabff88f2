// l2c_cuda.cu -- GB300 (sm_103a) implementation of the fast multipole
// Legendre<->Chebyshev transform behind the C ABI of include/l2c_cuda.h.
//
// One plan = one transform length N.  Everything the transform reads is built
// on the GPU at plan time and stays resident in HBM:
//   a[N], an[N], dn[(N+1)/2]   Lambda tables              (leg2cheb.c:758-818)
//   A[dir][3 N_b][18][18]      far-field blocks           (leg2cheb.c:924-995)
//   T[2][s][18]                Chebyshev Vandermonde      (leg2cheb.c:621-648)
// Execution of one batch of `count` vectors (leg2cheb.c:1299-1500):
//   gather      x = parity-ready contiguous copy (C2L: v_j = j u_j)
//   near band   y = out_in + near field                       (directM / directL)
//   leaf up     w[L-1] = leaf blocks * T_parity, both parities (step 1)
//   tree up     w[l] from w[l+1] through the binomial matrix  (step 2)
//   far         c = A w, every level in one launch             (step 3)
//   tree down   c[l+1] += B^T c[l]                             (step 4)
//   leaf down   out = scale (y + c[L-1] * T_parity^T)          (step 5 + scaling)
// FP64 is the scarce resource on this part (about 1 TFLOP/s against 74 TFLOP/s
// FP32), so the kernels are written to spend as few FP64 instructions per
// coefficient as the algorithm allows; index arithmetic is integer.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <functional>
#include <vector>

#include "../../include/l2c_cuda.h"
#include "l2c_lambda.h"
#include "l2c_ozaki.cuh"
#include "l2c_tc.cuh"

namespace {

constexpr int M = 18;
constexpr int MM = M * M;
constexpr int NTRI = (MM + M) / 2;
constexpr double TWO_OVER_PI = 0.63661977236758134308;  // 2/pi

// L2C output scale: 2/pi, halved for output 0.  Halving is exact, so one
// multiply by the selected factor gives the same double as the reference's two
// (val * 2/pi, then * 0.5 for j = 0) and costs one FP64 instruction per warp
// instead of two.
__host__ __device__ __forceinline__ double l2c_out_scale(long long j) {
  return j == 0 ? 0.5 * TWO_OVER_PI : TWO_OVER_PI;
}
constexpr double SQRT_PI = 1.77245385090551602729816;
constexpr double TWO_OVER_SQRT_PI = 1.12837916709551257390;

thread_local char g_err[512] = "";

void set_err(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return 0;                                                                        \
    }                                                                                  \
  } while (0)

__constant__ double c_lambda_int[256] = L2C_LAMBDA_INT_INIT;
__constant__ double c_binom_lower[NTRI] = L2C_BINOM_LOWER_INIT;
__constant__ double c_binom_upper[NTRI] = L2C_BINOM_UPPER_INIT;
__constant__ double c_xj[M];       // cos((i + 1/2) pi / M), host libm values
__constant__ double c_dct[M * M];  // cos(pi k (n + 1/2) / M), [k][n]
// Nodal form: interpolation from the Chebyshev points of a parent interval to
// those of its two children, B0 | B1 (row-major M x M each, leg2cheb.c:1076-1100)
__constant__ double c_lag_B[2 * M * M];

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start while the previous kernel on its stream is still
// running; pdl_wait() returns once that kernel has completed and its memory
// writes are visible (immediately when there is no such kernel), so a kernel
// reads or writes nothing the previous one touches before it.  pdl_trigger()
// lets the next kernel launch once every CTA of this one has passed it.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

// Launch options: programmatic stream serialization (the kernel may start
// while the previous kernel on its stream finishes, and must call pdl_wait()
// before it touches anything an earlier kernel writes or reads) and a
// scheduling priority (0: the stream's).
struct LaunchOpt {
  bool pdl = false;
  int prio = 0;
  LaunchOpt(bool pdl_) : pdl(pdl_) {}
  LaunchOpt(bool pdl_, int prio_) : pdl(pdl_), prio(prio_) {}
};

template <typename... KArgs, typename... Args>
void launch_k(LaunchOpt o, void (*kern)(KArgs...), dim3 grid, unsigned block, size_t smem,
              cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  unsigned n = 0;
  if (o.pdl) {
    at[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[n++].val.programmaticStreamSerializationAllowed = 1;
  }
  if (o.prio != 0) {
    at[n].id = cudaLaunchAttributePriority;
    at[n++].val.priority = o.prio;
  }
  cfg.attrs = at;
  cfg.numAttrs = n;
  (void)cudaLaunchKernelEx(&cfg, kern, args...);  // errors surface in cudaGetLastError()
}


// ---------------------------------------------------------------------------
// Tree bookkeeping (leg2cheb.c:125-150), as closed forms.
//   level l holds nb(l) = 2^(l+1) - 1 blocks and S(l) = 2 nb(l) slots;
//   blocks before level l: off(l) = 2^(l+1) - l - 2; slots before it: 2 off(l).
// Source slot j of level l is tree node j + 2; target slot t is node t.
// ---------------------------------------------------------------------------
__host__ __device__ inline size_t blocks_before(size_t l) { return ((size_t)2 << l) - l - 2; }
__host__ __device__ inline size_t slots_at(size_t l) { return ((size_t)4 << l) - 2; }

// ---------------------------------------------------------------------------
// Plan construction kernels
// ---------------------------------------------------------------------------

// a[i] = Lambda(i): table for i < 256; for i >= 256, Lambda(i) at multiples of 8
// and a[j] = a[j-1] - (a[j-1]/2)/j in between (leg2cheb.c:767-779).
__global__ void k_lambda_table(double *a, size_t N) {
  const size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t i0 = g * 8;
  if (i0 >= N) return;
  const size_t stop = i0 + 8 < N ? i0 + 8 : N;
  if (i0 < 256) {
    for (size_t i = i0; i < stop; i++) a[i] = c_lambda_int[i];
    return;
  }
  double v = l2c_lambda_eval((double)i0);
  a[i0] = v;
  for (size_t j = i0 + 1; j < stop; j++) {
    v = __dsub_rn(v, __ddiv_rn(__dmul_rn(0.5, v), (double)j));
    a[j] = v;
  }
}

// an[i] = 1/(a[i] (2 i^2 + i)), an[0] = 2/sqrt(pi); dn[i] = a[i-1]/(2 i), dn[0] = 0
// (leg2cheb.c:781-795).
__global__ void k_c2l_tables(const double *__restrict__ a, double *an, double *dn, size_t N) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < N)
    an[i] = (i == 0) ? TWO_OVER_SQRT_PI
                     : __ddiv_rn(1.0, __dmul_rn(a[i], (double)(2 * i * i + i)));
  if (i < (N + 1) / 2) dn[i] = (i == 0) ? 0.0 : __ddiv_rn(a[i - 1], (double)(2 * i));
}

// Shift-invariant factor Lambda((y-x)/2) of level l and offset q - p (block 0,
// p = 0), filled persymmetrically as the reference does (leg2cheb.c:948-955):
// computed where j < M - i, mirrored to (M-1-j, M-1-i).
__global__ void k_assemble_f0(double *f0, size_t L, size_t s) {
  const int l = blockIdx.x >> 1, q = blockIdx.x & 1;
  const int i = threadIdx.x / M, j = threadIdx.x % M;
  if (threadIdx.x >= MM || j >= M - i) return;
  const size_t hl = (size_t)1 << (L - l - 1);
  const size_t h = s * hl;
  const double hd = (double)h;
  const size_t x0 = h;                                // 2*(i0 + 0*h) + h with i0 = 0
  const size_t y0 = 2 * (2 * s * hl + q * h) + h;     // 2*(j0 + q*h) + h
  const double x = __dadd_rn((double)x0, __dmul_rn(c_xj[i], hd));
  const double y = __dadd_rn((double)y0, __dmul_rn(c_xj[j], hd));
  const double m0 = l2c_lambda_eval(__dmul_rn(__dsub_rn(y, x), 0.5));
  double *F = f0 + (size_t)blockIdx.x * MM;
  F[i * M + j] = m0;
  F[(M - 1 - j) * M + (M - 1 - i)] = m0;
}

// One far-field block per CTA: blockIdx.x = 3 g + r, g = global block index,
// r over (q,p) = (0,0), (1,0), (1,1).  Samples the kernel on the 18x18 Chebyshev
// grid (leg2cheb.c:924-972) and, in the modal form, converts it with a 2D
// DCT-II, A = (4/M^2) C F C^T with row 0 and column 0 halved (dct.c:582-598);
// the nodal form keeps the samples.
__global__ void __launch_bounds__(MM) k_assemble_A(const double *__restrict__ f0, double *A_l2c,
                                                   double *A_c2l, size_t L, size_t s, int nodal) {
  __shared__ double sF1[MM];
  __shared__ double sF[MM];
  __shared__ double sT[MM];
  const size_t g = blockIdx.x / 3;
  const int r = blockIdx.x % 3;
  const int q = r == 0 ? 0 : 1, p = r == 2 ? 1 : 0;
  size_t l = 0;
  while (l + 1 < L && blocks_before(l + 1) <= g) l++;
  const size_t b = g - blocks_before(l);
  const size_t hl = (size_t)1 << (L - l - 1);
  const size_t h = s * hl;
  const double hd = (double)h;
  const size_t i0 = 2 * b * s * hl, j0 = i0 + 2 * s * hl;
  const double x0 = (double)(2 * (i0 + p * h) + h);
  const double y0 = (double)(2 * (j0 + q * h) + h);
  const int t = threadIdx.x;
  const int i = t / M, j = t % M;
  // Lambda((x+y)/2), symmetric fill from (min, max) (leg2cheb.c:956-963)
  {
    const int lo = i < j ? i : j, hi = i < j ? j : i;
    const double x = __dadd_rn(x0, __dmul_rn(c_xj[lo], hd));
    const double y = __dadd_rn(y0, __dmul_rn(c_xj[hi], hd));
    sF1[t] = l2c_lambda_eval(__dmul_rn(__dadd_rn(x, y), 0.5));
  }
  __syncthreads();
  const double fpq = f0[((size_t)l * 2 + (q - p)) * MM + t];
  const double x = __dadd_rn(x0, __dmul_rn(c_xj[i], hd));
  const double y = __dadd_rn(y0, __dmul_rn(c_xj[j], hd));
  for (int dir = 0; dir < 2; dir++) {
    double *Ad = dir == 0 ? A_l2c : A_c2l;
    if (Ad == nullptr) continue;
    if (dir == 0) {
      sF[t] = __dmul_rn(fpq, sF1[t]);
    } else {
      const double xy = __dadd_rn(x, y);
      double den = __dmul_rn(sF1[t], xy);
      den = __dmul_rn(den, __dadd_rn(xy, 1.0));
      den = __dmul_rn(den, __dadd_rn(__dsub_rn(x, y), 1.0));
      sF[t] = __dmul_rn(2.0, __ddiv_rn(fpq, den));
    }
    if (nodal) {  // the nodal form keeps the kernel samples (leg2cheb.c:938, 973)
      Ad[(size_t)blockIdx.x * MM + t] = sF[t];
      continue;
    }
    __syncthreads();
    // rows: sT[i][k] = sum_n F[i][n] C[k][n]
    {
      const int k = j;
      double acc = 0.0;
#pragma unroll
      for (int n = 0; n < M; n++) acc = fma(sF[i * M + n], c_dct[k * M + n], acc);
      sT[i * M + k] = acc;
    }
    __syncthreads();
    // columns: out[k1][k2] = sum_i C[k1][i] sT[i][k2]
    {
      const int k1 = i, k2 = j;
      double acc = 0.0;
#pragma unroll
      for (int n = 0; n < M; n++) acc = fma(c_dct[k1 * M + n], sT[n * M + k2], acc);
      acc *= (1.0 / 81.0);
      if (k1 == 0) acc *= 0.5;
      if (k2 == 0) acc *= 0.5;
      Ad[(size_t)blockIdx.x * MM + t] = acc;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Execution kernels.  Batch layout: vector v of `count`; caller arrays use
// (dist, stride); internal arrays are contiguous per vector (x, y: N each;
// w, c: 2 parities x 2 N_b slots x M).
// ---------------------------------------------------------------------------

// n 2^e as a double, exactly (0 <= n < 2^53), by bit construction: integer
// instructions instead of a conversion on the FP64 pipe.
__device__ __forceinline__ double dyadic(unsigned long long n, int e) {
  const int lz = __clzll((long long)n);
  const unsigned long long frac = (n << ((lz + 1) & 63)) >> 12;  // bits after the leading one
  const unsigned long long bits = ((unsigned long long)(1023 + 63 - lz + e) << 52) | frac;
  return n == 0 ? 0.0 : __longlong_as_double((long long)bits);
}

struct Geo {
  long long N, s, h, nL, L, K, slots, leaf_base, count, dist, stride;
};

// Each phase is written once as a per-item device function working on one
// vector's arrays; the uniform-batch kernels below and the ragged-batch kernels
// (one launch over vectors of different N) both call them.

// x[j] = in[j stride], premultiplied by j (j >= 2) for C2L (leg2cheb.c:1325-1335).
__device__ __forceinline__ void gather_item(const double *__restrict__ in, double *__restrict__ x,
                                            long long stride, int c2l, long long j) {
  double u = in[j * stride];
  if (c2l && j >= 2) u = u * dyadic((unsigned long long)j, 0);
  x[j] = u;
}

__global__ void k_gather(const double *__restrict__ in, double *__restrict__ x, Geo g, int c2l) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.count * g.N) return;
  const long long v = idx / g.N, j = idx - v * g.N;
  gather_item(in + v * g.dist, x + v * g.N, g.stride, c2l, j);
}

// Near-field band, one output per thread.  For output j in block b = min(j/h, nL-1)
// the band covers sources j + 2k < lim = min((b+2) h, N), with weight w(k, j):
//   L2C: w = a[k] a[j+k]                                         (leg2cheb.c:236-302)
//   C2L: w = sqrt(pi) an[j] (k = 0),  -(dn[k] an[j+k]) (k >= 1)  (leg2cheb.c:392-459)
// and y = out_in + sum_k w(k, j) x[j+2k], accumulated by FMA from k = 0.
// The weight is formed on the fly (one DMUL + one DFMA per term) or read from a
// table built at plan time (one DFMA per term, same bits; see k_near_weights).
__device__ __forceinline__ double near_weight(int c2l, long long k, long long j,
                                              const double *__restrict__ a,
                                              const double *__restrict__ an,
                                              const double *__restrict__ dn) {
  if (!c2l) return a[k] * a[j + k];
  if (k == 0) return SQRT_PI * an[j];
  return -(dn[k] * an[j + k]);
}

// Number of band terms of output position i of block b at source offset k
// (the table layout of the precomputed weights, block-major, then k, then i).
__device__ __forceinline__ long long band_count(long long k, long long b, const Geo &g) {
  if (b < g.nL - 1) return k < g.s ? g.h : 2 * g.h - 2 * k;
  const long long c = g.N - (g.nL - 1) * g.h - 2 * k;
  return c > 0 ? c : 0;
}

// Band sum of output j for VB vectors (x rows g.N apart), two accumulator sets
// (even and odd k) to halve the dependent FP64 chain.  W: precomputed weights of
// this plan (or nullptr: weights formed on the fly).
template <int VB>
__device__ __forceinline__ void near_sums(const double *__restrict__ xv, long long xstride,
                                          const double *__restrict__ a,
                                          const double *__restrict__ an,
                                          const double *__restrict__ dn,
                                          const double *__restrict__ W, const Geo &g, int c2l,
                                          long long j, double *res) {
  long long b = j / g.h;
  if (b > g.nL - 1) b = g.nL - 1;
  long long lim = (b + 2) * g.h;
  if (lim > g.N) lim = g.N;
  const long long nk = (lim - j + 1) / 2;  // terms k = 0 .. nk-1
  double acc0[VB], acc1[VB];
#pragma unroll
  for (int u = 0; u < VB; u++) acc0[u] = acc1[u] = 0.0;
  if (W == nullptr) {
    long long k = 0;
    for (; k + 1 < nk; k += 2) {
      const double w0 = near_weight(c2l, k, j, a, an, dn);
      const double w1 = near_weight(c2l, k + 1, j, a, an, dn);
#pragma unroll
      for (int u = 0; u < VB; u++) {
        acc0[u] = fma(w0, xv[u * xstride + 2 * k], acc0[u]);
        acc1[u] = fma(w1, xv[u * xstride + 2 * k + 2], acc1[u]);
      }
    }
    if (k < nk) {
      const double w0 = near_weight(c2l, k, j, a, an, dn);
#pragma unroll
      for (int u = 0; u < VB; u++) acc0[u] = fma(w0, xv[u * xstride + 2 * k], acc0[u]);
    }
  } else {
    const long long i = j - b * g.h;
    const double *Wb = W + b * (3 * g.s * g.s + g.s);
    long long off = 0, k = 0;
    // four terms per iteration, all loads issued before the FMAs, to keep
    // enough weight loads in flight to cover DRAM latency
    for (; k + 3 < nk; k += 4) {
      const long long o1 = off + band_count(k, b, g);
      const long long o2 = o1 + band_count(k + 1, b, g);
      const long long o3 = o2 + band_count(k + 2, b, g);
      const double w0 = Wb[off + i], w1 = Wb[o1 + i], w2 = Wb[o2 + i], w3 = Wb[o3 + i];
      double xa[VB][4];
#pragma unroll
      for (int u = 0; u < VB; u++)
#pragma unroll
        for (int r = 0; r < 4; r++) xa[u][r] = xv[u * xstride + 2 * (k + r)];
#pragma unroll
      for (int u = 0; u < VB; u++) {
        acc0[u] = fma(w0, xa[u][0], acc0[u]);
        acc1[u] = fma(w1, xa[u][1], acc1[u]);
        acc0[u] = fma(w2, xa[u][2], acc0[u]);
        acc1[u] = fma(w3, xa[u][3], acc1[u]);
      }
      off = o3 + band_count(k + 3, b, g);
    }
    for (; k + 1 < nk; k += 2) {
      const long long off1 = off + band_count(k, b, g);
      const double w0 = Wb[off + i], w1 = Wb[off1 + i];
#pragma unroll
      for (int u = 0; u < VB; u++) {
        acc0[u] = fma(w0, xv[u * xstride + 2 * k], acc0[u]);
        acc1[u] = fma(w1, xv[u * xstride + 2 * k + 2], acc1[u]);
      }
      off = off1 + band_count(k + 1, b, g);
    }
    if (k < nk) {
      const double w0 = Wb[off + i];
#pragma unroll
      for (int u = 0; u < VB; u++) acc0[u] = fma(w0, xv[u * xstride + 2 * k], acc0[u]);
    }
  }
#pragma unroll
  for (int u = 0; u < VB; u++) res[u] = acc0[u] + acc1[u];
}

// VB vectors per thread: the weight of each term is formed (or loaded) once and
// used for VB vectors.  blockIdx.x enumerates (output tile, vector group) with
// the tile index fastest.  y = out_in + band.
template <int VB>
__global__ void __launch_bounds__(256, VB == 1 ? 5 : VB == 2 ? 4 : 2)
    k_near(const double *__restrict__ x, const double *out, double *__restrict__ y,
           const double *__restrict__ a, const double *__restrict__ an,
           const double *__restrict__ dn, const double *__restrict__ W, Geo g, int c2l,
           long long jbeg) {
  pdl_wait();
  pdl_trigger();
  const long long ntile = (g.N - jbeg + blockDim.x - 1) / blockDim.x;
  const long long nblk = ntile * (g.count / VB);
  for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {  // grid may be smaller
    const long long tile = blk % ntile, vg = blk / ntile;
    const long long j = jbeg + tile * blockDim.x + threadIdx.x;
    if (j >= g.N) continue;
    const long long v0 = vg * VB;
    double res[VB];
    near_sums<VB>(x + v0 * g.N + j, g.N, a, an, dn, W, g, c2l, j, res);
#pragma unroll
    for (int u = 0; u < VB; u++)
      y[(v0 + u) * g.N + j] = out[(v0 + u) * g.dist + j * g.stride] + res[u];
  }
}

// Band of the blocks b < nL-1 in pairs: one thread forms outputs i and h-1-i
// of block b for VB vectors.  Their term counts add up to 3h/2 + 1 for every
// i, so all lanes of a warp run the same number of FP64 instructions (one
// output per thread leaves up to half the lanes idle at the end of the loop).
// Terms are accumulated in order k = 0, 1, ... into one FMA chain per output
// (the FP64 pipe, not its latency, bounds this loop).  Threads past the pairs
// of a vector group take the outputs of the last (ragged) block one each, in
// the same launch, so that block runs beside the others.  Register bound:
// three 256-thread CTAs per SM (80 registers at VB = 8, a few spilled);
// the extra resident warps more than pay for the spills (256 x 16384, s = 16:
// 0.573 -> 0.531 ms per L2C + C2L alone, and room for the far-field chain
// beside it).
template <int VB>
__global__ void __launch_bounds__(256, 3)
    k_near_pair(const double *__restrict__ x, const double *out, double *__restrict__ y,
                const double *__restrict__ a, const double *__restrict__ an,
                const double *__restrict__ dn, const double *__restrict__ W, Geo g, int c2l) {
  pdl_wait();
  pdl_trigger();
  const long long half = g.h >> 1, npair = (g.nL - 1) * half, jlast = (g.nL - 1) * g.h;
  const long long per_vg = npair + (g.N - jlast), nitem = per_vg * (g.count / VB);
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < nitem;
       idx += (long long)gridDim.x * blockDim.x) {  // the grid may be smaller than the work
    const long long vg = idx / per_vg;
    const long long r = idx - vg * per_vg;
    if (r >= npair) {
      const long long j = jlast + (r - npair), v0 = vg * VB;
      double res[VB];
      near_sums<VB>(x + v0 * g.N + j, g.N, a, an, dn, W, g, c2l, j, res);
#pragma unroll
      for (int u = 0; u < VB; u++)
        y[(v0 + u) * g.N + j] = out[(v0 + u) * g.dist + j * g.stride] + res[u];
      continue;
    }
    const long long b = r / half, i = r - b * half;
    const long long jA = b * g.h + i, jB = b * g.h + g.h - 1 - i, lim = (b + 2) * g.h;
    const long long nkA = (lim - jA + 1) >> 1, total = nkA + ((lim - jB + 1) >> 1);
    const double *xv = x + vg * VB * g.N;
    const double *Wb = W ? W + b * (3 * g.s * g.s + g.s) : nullptr;
    double acc[VB], resA[VB];
#pragma unroll
    for (int u = 0; u < VB; u++) acc[u] = resA[u] = 0.0;
    for (long long t = 0; t < total; t++) {
      const bool second = t >= nkA;
      const long long j = second ? jB : jA, k = second ? t - nkA : t;
      double wt;
      if (Wb) {
        // offset of term k in the block's table: k h for k < s, then rows of 2h - 2k'
        const long long off =
            k < g.s ? k * g.h : 4 * g.s * k - k * k + k - g.s * g.s - g.s;
        wt = Wb[off + (j - b * g.h)];
      } else {
        wt = near_weight(c2l, k, j, a, an, dn);
      }
#pragma unroll
      for (int u = 0; u < VB; u++) acc[u] = fma(wt, xv[u * g.N + j + 2 * k], acc[u]);
      if (t == nkA - 1) {
#pragma unroll
        for (int u = 0; u < VB; u++) {
          resA[u] = acc[u];
          acc[u] = 0.0;
        }
      }
    }
    const long long v0 = vg * VB;
#pragma unroll
    for (int u = 0; u < VB; u++) {
      y[(v0 + u) * g.N + jA] = out[(v0 + u) * g.dist + jA * g.stride] + resA[u];
      y[(v0 + u) * g.N + jB] = out[(v0 + u) * g.dist + jB * g.stride] + acc[u];
    }
  }
}

// Plan time: the band weights of every output, in the layout k_near reads.
__global__ void k_near_weights(double *__restrict__ W, const double *__restrict__ a,
                               const double *__restrict__ an, const double *__restrict__ dn,
                               Geo g, int c2l) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j >= g.N) return;
  long long b = j / g.h;
  if (b > g.nL - 1) b = g.nL - 1;
  long long lim = (b + 2) * g.h;
  if (lim > g.N) lim = g.N;
  const long long i = j - b * g.h;
  double *Wb = W + b * (3 * g.s * g.s + g.s);
  long long off = 0;
  for (long long k = 0; j + 2 * k < lim; k++) {
    Wb[off + i] = near_weight(c2l, k, j, a, an, dn);
    off += band_count(k, b, g);
  }
}

// Size of the weight table: (nL - 1) full blocks of 3 s^2 + s entries and the
// last (ragged) block.
inline size_t near_table_size(size_t N, size_t s) {
  const size_t h = 2 * s, nL = N / h, rest = N - (nL - 1) * h;
  size_t n = (nL - 1) * (3 * s * s + s);
  for (size_t k = 0; 2 * k < rest; k++) n += rest - 2 * k;
  return n;
}

// Band of one vector with register windows (full blocks b < nL-1).  Output
// j = b h + 2 i' + p sums, over sources m' = i' .. 2s-1 of block b and parity
// p, w(k, j) x[b h + 2 m' + p] with k = m' - i', where w = lo[k] hi[j + k]
// (L2C: a[k] a[j+k]; C2L: -(dn[k] an[j+k]), with -sqrt(pi) standing for dn[0],
// which gives the k = 0 term sqrt(pi) an[j] exactly) and j + k = b h + p + i'
// + m'.  A thread owns a row group, up to 4 consecutive rows i'0 .. i'0+3 of
// one parity: at source m' every row reads the same x, and as m' advances by
// one the rows' lo values shift down one row and their hi values up one row,
// so each step loads one x, one lo and one hi value for 4 DMUL + 4 DFMA (the
// per-output kernel loads all three per term).  The lanes of a warp take the
// same row group of consecutive blocks, so they run the same trip count.
// Terms are summed in order of k into one FMA chain from zero; y = out_in +
// sum.  TAB: weights from the dense per-block table of k_band_tile_weights
// (W'[b][p][m'][i'], the row group's four at one m' contiguous; the same
// products, the same bits; that loop is unrolled so that the table loads of
// several steps are in flight together).
template <bool TAB>
__device__ __forceinline__ void near_rows_group(const double *__restrict__ xb,
                                                const double *__restrict__ lo,
                                                const double *__restrict__ hi,
                                                const double *__restrict__ Wg, long long hbase,
                                                const Geo &g, int c2l, int p, int ip0, int R,
                                                double (&acc)[4]) {
  const int s2 = 2 * (int)g.s;
  auto lo_at = [&](int k) -> double { return c2l && k == 0 ? -SQRT_PI : lo[k]; };
  double wl[4], wh[4];  // row r: lo[m' - i'0 - r], hi[hbase + i'0 + r + m']
#pragma unroll
  for (int r = 0; r < 4; r++) {
    acc[r] = 0.0;
    wl[r] = 0.0;
    wh[r] = TAB || r >= R ? 0.0 : hi[hbase + ip0 + r + ip0];
  }
#pragma unroll(TAB ? 8 : 1)
  for (int mp = ip0; mp < s2; mp++) {
    const int t = mp - ip0;  // rows r <= t have a term at this m'
    double wt[4];
    if (TAB) {
      // the group's four weights at m' (16-byte aligned when s is even: the
      // table's rows are s doubles long)
      const double *wq = Wg + (long long)mp * g.s;
      if ((g.s & 1) == 0) {
        const double2 q0 = __ldg(reinterpret_cast<const double2 *>(wq));
        const double2 q1 = __ldg(reinterpret_cast<const double2 *>(wq) + 1);
        wt[0] = q0.x;
        wt[1] = q0.y;
        wt[2] = q1.x;
        wt[3] = q1.y;
      } else {
#pragma unroll
        for (int r = 0; r < 4; r++) wt[r] = __ldg(wq + r);
      }
    } else {
      // shift the windows to m' and bring in row 0's lo and row R-1's hi
#pragma unroll
      for (int r = 3; r > 0; r--) wl[r] = wl[r - 1];
      wl[0] = lo_at(t);
      if (t > 0) {
#pragma unroll
        for (int r = 0; r < 3; r++) wh[r] = wh[r + 1];
        if (R == 4) {
          wh[3] = hi[hbase + ip0 + 3 + mp];
        } else {
#pragma unroll
          for (int r = 0; r < 3; r++)
            if (r == R - 1) wh[r] = hi[hbase + ip0 + r + mp];
        }
      }
    }
    const double xv = xb[2 * mp + p];
#pragma unroll
    for (int r = 0; r < 4; r++)
      if (r <= t && r < R) {
        const double w = TAB ? wt[r] : c2l ? -(wl[r] * wh[r]) : wl[r] * wh[r];
        acc[r] = fma(w, xv, acc[r]);
      }
  }
}

// Item it of a vector's band with register windows: the last (ragged) block
// first, one output per thread (k_near's sums, weights formed on the fly),
// then (parity, row group, block) with the block fastest.  x, out, y: the
// vector's arrays (out with g.stride); a, an, dn: its Lambda tables; W: its
// dense weight table (k_band_tile_weights) or nullptr.
template <bool TAB>
__device__ __forceinline__ void near_rows_item(const double *__restrict__ x, const double *out,
                                               double *__restrict__ y,
                                               const double *__restrict__ a,
                                               const double *__restrict__ an,
                                               const double *__restrict__ dn,
                                               const double *__restrict__ W, const Geo &g,
                                               int c2l, long long it) {
  const long long nb = g.nL - 1, jlast = nb * g.h, ntail = g.N - jlast;
  if (it < ntail) {
    const long long j = jlast + it;
    double res[1];
    near_sums<1>(x + j, g.N, a, an, dn, nullptr, g, c2l, j, res);
    y[j] = out[j * g.stride] + res[0];
    return;
  }
  it -= ntail;
  const long long G = (g.s + 3) / 4;  // row groups per parity
  const long long pg = it / nb, b = it - pg * nb;
  const int p = (int)(pg / G), gi = (int)(pg % G), ip0 = 4 * gi;
  const int R = (int)g.s - ip0 < 4 ? (int)g.s - ip0 : 4;
  double acc[4];
  near_rows_group<TAB>(x + b * g.h, c2l ? dn : a, c2l ? an : a,
                       TAB ? W + ((b * 2 + p) * 2 * g.s) * g.s + ip0 : nullptr, b * g.h + p, g,
                       c2l, p, ip0, R, acc);
#pragma unroll
  for (int r = 0; r < 4; r++)
    if (r < R) {
      const long long j = b * g.h + 2 * (ip0 + r) + p;
      y[j] = out[j * g.stride] + acc[r];
    }
}

// Items of a vector's band (near_rows_item).
__host__ __device__ inline long long near_rows_items(const Geo &g) {
  return (g.N - (g.nL - 1) * g.h) + (g.nL - 1) * 2 * ((g.s + 3) / 4);
}

template <bool TAB>
__global__ void __launch_bounds__(256) k_near_rows(const double *__restrict__ x, const double *out,
                                                   double *__restrict__ y,
                                                   const double *__restrict__ a,
                                                   const double *__restrict__ an,
                                                   const double *__restrict__ dn,
                                                   const double *__restrict__ W, Geo g, int c2l) {
  pdl_wait();
  pdl_trigger();
  const long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (it < near_rows_items(g)) near_rows_item<TAB>(x, out, y, a, an, dn, W, g, c2l, it);
}

// Whether a single vector's band takes k_near_rows: at least 64 CTAs of row
// items (any = true: any size).  Its sums are chains of up to 2s dependent
// FMAs, so a vector with fewer blocks is bound by their latency and takes the
// per-output kernel, whose two chains per output are half as long and whose
// threads are four times as many.
inline bool near_rows_ok(long long s, long long nL, long long count, bool any = false) {
  return count == 1 && s >= 1 && nL >= 2 &&
         (any || (nL - 1) * 2 * ((s + 3) / 4) >= 64 * 256);
}

// Step 1: leaf node t in [2, 2^(L+1)) of parity sg: w = sum_i x[t h + 2i + sg] T_sg[i][m].
// xv: this vector's x; wv: this vector's w (2 parities x slots x M).
__device__ __forceinline__ void leaf_up_item(const double *__restrict__ xv,
                                             const double *__restrict__ T,
                                             double *__restrict__ wv, const Geo &g,
                                             long long node, int sg, int m) {
  const long long base = (node + 2) * g.h + sg;
  const double *Ts = T + (size_t)sg * g.s * M + m;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  long long iend = (g.N - base + 1) / 2;  // number of i with base + 2i < N
  if (iend > g.s) iend = g.s;
  long long i = 0;
  for (; i + 3 < iend; i += 4) {
#pragma unroll
    for (int r = 0; r < 4; r++) acc[r] = fma(xv[base + 2 * (i + r)], Ts[(i + r) * M], acc[r]);
  }
  for (; i < iend; i++) acc[0] = fma(xv[base + 2 * i], Ts[i * M], acc[0]);
  wv[((long long)sg * g.slots + g.leaf_base + node) * M + m] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

// One thread per (vector, node, parity, m).
__global__ void __launch_bounds__(288) k_leaf_up(const double *__restrict__ x,
                                                 const double *__restrict__ T,
                                                 double *__restrict__ w, Geo g) {
  pdl_wait();
  pdl_trigger();
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long per_vec = g.K * 2 * M;
  if (idx >= g.count * per_vec) return;
  const long long v = idx / per_vec;
  long long rem = idx - v * per_vec;
  const long long node = rem / (2 * M);
  rem -= node * 2 * M;
  leaf_up_item(x + v * g.N, T, w + v * 2 * g.slots * M, g, node, (int)(rem / M), (int)(rem % M));
}

// Step 2, one level: parent slot j of level l from child slots 2j+2, 2j+3 of level
// l+1 through the compact lower binomial matrix (leg2cheb.c:537-602):
//   b[m] = sum_{i<=m} B[m][i] x0[i] + sum_{i<=m} (-1)^(m+i) B[m][i] x1[i],
// the +/- parity combination of the reference written as two independent FMA
// chains.  A CTA takes TREE_TILE parents: their 36 child coefficients are staged
// in shared memory with coalesced loads (children of consecutive parents are
// contiguous), then warp m computes row m for every parent of the tile, so loop
// lengths are warp-uniform and no load sits inside the FMA loop.
constexpr int TREE_TILE = 32;
constexpr int TREE_PAD = 2 * M + 1;  // padded row of staged children (bank spread)

// Transfer matrices in shared memory: modal, the compact lower (upward) or
// upper (downward) binomial matrix, NTRI doubles; nodal, B0 | B1 (2 M^2).
template <bool NODAL>
__host__ __device__ constexpr int tree_mat_size() {
  return NODAL ? 2 * MM : NTRI;
}
template <bool NODAL, bool UP>
__device__ __forceinline__ void load_tree_mat(double *sB) {
  for (int t = threadIdx.x; t < tree_mat_size<NODAL>(); t += blockDim.x)
    sB[t] = NODAL ? c_lag_B[t] : UP ? c_binom_lower[t] : c_binom_upper[t];
}

// Modal upward transfer, first half (leg2cheb.c:537-602): the children x0, x1
// of a parent become z+ = x0 + S x1 and z- = x0 - S x1 in place (S = diag(1,
// -1, 1, ...)), element i of the pair.  Nodal: nothing.
template <bool NODAL>
__device__ __forceinline__ void zpm_item(double *x0, double *x1, int i) {
  if (NODAL) return;
  const double a = x0[i], b = (i & 1) ? -x1[i] : x1[i];
  x0[i] = a + b;
  x1[i] = a - b;
}

// Row m of a parent from its two children.  Modal: the lower binomial row
// times z+ (even m) or z- (odd m), the children after zpm_item (leg2cheb.c:
// 537-602: 36 adds and 171 FMAs per parent); nodal: column m of B0 and of B1,
// out = B0^T x0 + B1^T x1 (leg2cheb.c:1401-1416).
template <bool NODAL>
__device__ __forceinline__ void row_up(const double *sB, const double *x0, const double *x1, int m,
                                       double &out) {
  double s0 = 0.0, s1 = 0.0;
  if (NODAL) {
    for (int i = 0; i < M; i++) {
      s0 = fma(sB[i * M + m], x0[i], s0);
      s1 = fma(sB[MM + i * M + m], x1[i], s1);
    }
  } else {
    const double *Bm = sB + m * (m + 1) / 2, *z = (m & 1) ? x1 : x0;
    int i = 0;
    for (; i + 1 <= m; i += 2) {  // two chains (even, odd i) halve the latency
      s0 = fma(Bm[i], z[i], s0);
      s1 = fma(Bm[i + 1], z[i + 1], s1);
    }
    if (i <= m) s0 = fma(Bm[i], z[i], s0);
  }
  out = s0 + s1;
}

// Increments d0, d1 of row i of the two children of parent xp.  Modal: the
// compact upper binomial row, se/so over the columns of equal/opposite parity
// to the row, d0 = se + so, d1 = se - so (leg2cheb.c:603-618); nodal: row i of
// B0 and of B1 (leg2cheb.c:1450-1464).
template <bool NODAL>
__device__ __forceinline__ void row_down(const double *sB, const double *xp, int i, double &d0,
                                         double &d1) {
  if (NODAL) {
    double a = 0.0, b = 0.0;
    for (int j = 0; j < M; j++) {
      a = fma(sB[i * M + j], xp[j], a);
      b = fma(sB[MM + i * M + j], xp[j], b);
    }
    d0 = a;
    d1 = b;
    return;
  }
  const double *Bu = sB + i * M - i * (i - 1) / 2 - i;  // Bu[j] = row i, column j
  double se = 0.0, so = 0.0;
  int j = i;
  for (; j + 1 < M; j += 2) {
    se = fma(Bu[j], xp[j], se);
    so = fma(Bu[j + 1], xp[j + 1], so);
  }
  if (j < M) se = fma(Bu[j], xp[j], se);
  d0 = se + so;
  d1 = se - so;
}

// One tile: child[p] points at the 2M child coefficients of item p, par[p] at
// its M parent coefficients (nullptr: no item).
template <bool NODAL = false>
__device__ __forceinline__ void tree_up_tile(const double *const *child, double *const *par,
                                             const double *sB, double *sx) {
  for (int e = threadIdx.x; e < TREE_TILE * 2 * M; e += blockDim.x) {
    const int p = e / (2 * M), q = e - p * 2 * M;
    sx[p * TREE_PAD + q] = par[p] ? child[p][q] : 0.0;
  }
  __syncthreads();
  if (!NODAL) {
    for (int e = threadIdx.x; e < TREE_TILE * M; e += blockDim.x) {
      const int p = e / M, i = e - p * M;
      zpm_item<NODAL>(sx + p * TREE_PAD, sx + p * TREE_PAD + M, i);
    }
    __syncthreads();
  }
  const int m = threadIdx.x >> 5, p = threadIdx.x & 31;
  if (m >= M || par[p] == nullptr) return;
  const double *x0 = sx + p * TREE_PAD, *x1 = x0 + M;
  double out;
  row_up<NODAL>(sB, x0, x1, m, out);
  par[p][m] = out;
}

// blockDim = 32 * M; items (vector * 2 + parity, parent slot) in TREE_TILE tiles.
template <bool NODAL>
__global__ void __launch_bounds__(32 * M) k_tree_up(double *w, Geo g, long long parent_base,
                                                    long long child_base, long long nparent) {
  pdl_wait();
  pdl_trigger();
  __shared__ double sB[tree_mat_size<NODAL>()];
  __shared__ double sx[TREE_TILE * TREE_PAD];
  __shared__ const double *child[TREE_TILE];
  __shared__ double *par[TREE_TILE];
  load_tree_mat<NODAL, true>(sB);
  if (threadIdx.x < TREE_TILE) {
    const long long item = (long long)blockIdx.x * TREE_TILE + threadIdx.x;
    const long long nitem = g.count * 2 * nparent;
    const long long vs = item / nparent, jp = item - vs * nparent;
    child[threadIdx.x] = w + (vs * g.slots + child_base + 2 * jp + 2) * M;
    par[threadIdx.x] = item < nitem ? w + (vs * g.slots + parent_base + jp) * M : nullptr;
  }
  __syncthreads();
  tree_up_tile<NODAL>(child, par, sB, sx);
}

// Two-stage sweeps for deep trees.  Every tree level costs a launch and a chain
// of dependent FP64 operations (64 cycles each on this part) however little work
// it holds, so the L-1 levels of a sweep are not launched one by one:
//   subtree kernels: one CTA per (vector, parity, subtree root r at level l0)
//     runs the d = L-1-l0 levels below l0 in shared memory;
//   top kernels: one CTA per (vector, parity) runs the levels above lt <= l0
//     in shared memory; levels between lt and l0 (only for very deep trees) use
//     the tiled per-level kernels above.
// Node index t at level l covers 2^k nodes [t 2^k, (t+1) 2^k) at level l+k.
// Source slots of level l are nodes 2..2^(l+2)-1 (slot = node - 2), target
// slots are nodes 0..2^(l+2)-3.
constexpr int SUB_PAD = M + 1;  // padded node stride in shared memory

// Upward, levels L-1 .. l0 of one subtree.  blockIdx.x = vs * R + r, R = 2^(l0+2).
// Dynamic shared memory: (2^(d+1) - 1) nodes of SUB_PAD doubles.
template <bool NODAL>
__global__ void __launch_bounds__(32 * M) k_up_sub(double *w, Geo g, int l0, int d) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ double sm[];
  __shared__ double sB[tree_mat_size<NODAL>()];
  load_tree_mat<NODAL, true>(sB);
  const long long R = 4LL << l0;
  const long long vs = blockIdx.x / R, r = blockIdx.x - vs * R;
  double *ws = w + vs * g.slots * M;
  // leaf level of the subtree
  const int nl = 1 << d;
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
    const int p = e / M, m = e - p * M;
    const long long t = r * nl + p;
    sm[p * SUB_PAD + m] = t >= 2 ? ws[(g.leaf_base + t - 2) * M + m] : 0.0;
  }
  __syncthreads();
  double *child = sm;
  for (int k = 1; k <= d; k++) {
    const int np = nl >> k, lg = d - k;  // np = 2^lg parents
    double *par = child + 2 * np * SUB_PAD;
    const int l = g.L - 1 - k;
    const long long base = 2 * (long long)blocks_before((size_t)l);
    // (parent, row) items packed densely over the CTA: a warp FP64 instruction
    // costs the same with idle lanes, so narrow levels use few, full warps
    if (!NODAL) {
      for (int it = threadIdx.x; it < np * M; it += blockDim.x) {
        const int p = it & (np - 1), i = it >> lg;
        zpm_item<NODAL>(child + 2 * p * SUB_PAD, child + (2 * p + 1) * SUB_PAD, i);
      }
      __syncthreads();
    }
    for (int it = threadIdx.x; it < np * M; it += blockDim.x) {
      const int p = it & (np - 1), m = it >> lg;
      const long long u = r * np + p;
      if (u < 2) continue;
      double out;
      row_up<NODAL>(sB, child + 2 * p * SUB_PAD, child + (2 * p + 1) * SUB_PAD, m, out);
      par[p * SUB_PAD + m] = out;
      ws[(base + u - 2) * M + m] = out;
    }
    __syncthreads();
    child = par;
  }
}

// Upward, levels lt-1 .. 0 of one (vector, parity) from level lt in global
// memory.  Dynamic shared memory: sum over l <= lt of 2^(l+2) nodes.
template <bool NODAL>
__global__ void __launch_bounds__(32 * M) k_up_top(double *w, Geo g, int lt) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ double sm[];
  __shared__ double sB[tree_mat_size<NODAL>()];
  load_tree_mat<NODAL, true>(sB);
  const long long vs = blockIdx.x;
  double *ws = w + vs * g.slots * M;
  // node t of level l at sm + (off(l) + t) * SUB_PAD, off(l) = 2^(l+2) - 4
  const long long nt = 4LL << lt;
  for (long long e = threadIdx.x; e < (nt - 2) * M; e += blockDim.x) {
    const long long j = e / M;
    const int m = (int)(e - j * M);
    sm[((nt - 4) + j + 2) * SUB_PAD + m] = ws[(2 * (long long)blocks_before((size_t)lt) + j) * M + m];
  }
  __syncthreads();
  for (int l = lt - 1; l >= 0; l--) {
    const int nn = 4 << l;  // nodes of level l; sources are nodes 2 .. nn-1
    double *par = sm + (nn - 4) * SUB_PAD, *child = sm + (2 * nn - 4) * SUB_PAD;
    const long long base = 2 * (long long)blocks_before((size_t)l);
    if (!NODAL) {
      for (int it = threadIdx.x; it < (nn - 2) * M; it += blockDim.x) {
        const int u = 2 + it % (nn - 2), i = it / (nn - 2);
        zpm_item<NODAL>(child + 2 * u * SUB_PAD, child + (2 * u + 1) * SUB_PAD, i);
      }
      __syncthreads();
    }
    for (int it = threadIdx.x; it < (nn - 2) * M; it += blockDim.x) {  // dense items
      const int u = 2 + it % (nn - 2), m = it / (nn - 2);
      double out;
      row_up<NODAL>(sB, child + 2 * u * SUB_PAD, child + (2 * u + 1) * SUB_PAD, m, out);
      par[u * SUB_PAD + m] = out;
      ws[(base + u - 2) * M + m] = out;
    }
    __syncthreads();
  }
}

// Downward, levels 0 .. lt of one (vector, parity): c[l+1] += B^T c[l] for
// l < lt, then levels 1..lt written back.  Dynamic shared memory as k_up_top.
template <bool NODAL>
__global__ void __launch_bounds__(32 * M) k_down_top(double *c, Geo g, int lt) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ double sm[];
  __shared__ double sB[tree_mat_size<NODAL>()];
  load_tree_mat<NODAL, false>(sB);
  const long long vs = blockIdx.x;
  double *cs = c + vs * g.slots * M;
  // target node t of level l at sm + (off(l) + t) * SUB_PAD; slots t < 2^(l+2)-2
  for (int l = 0; l <= lt; l++) {
    const long long nn = (4LL << l) - 2;
    const long long off = (4LL << l) - 4, base = 2 * (long long)blocks_before((size_t)l);
    for (long long e = threadIdx.x; e < nn * M; e += blockDim.x) {
      const long long t = e / M;
      const int m = (int)(e - t * M);
      sm[(off + t) * SUB_PAD + m] = cs[(base + t) * M + m];
    }
  }
  __syncthreads();
  for (int l = 0; l < lt; l++) {
    const int nn = (4 << l) - 2;
    double *par = sm + ((4LL << l) - 4) * SUB_PAD, *child = sm + ((8LL << l) - 4) * SUB_PAD;
    for (int it = threadIdx.x; it < nn * M; it += blockDim.x) {  // dense (target, row) items
      const int t = it % nn, i = it / nn;
      double d0, d1;
      row_down<NODAL>(sB, par + t * SUB_PAD, i, d0, d1);
      child[(2 * t) * SUB_PAD + i] += d0;
      child[(2 * t + 1) * SUB_PAD + i] += d1;
    }
    __syncthreads();
  }
  for (int l = 1; l <= lt; l++) {
    const long long nn = (4LL << l) - 2;
    const long long off = (4LL << l) - 4, base = 2 * (long long)blocks_before((size_t)l);
    for (long long e = threadIdx.x; e < nn * M; e += blockDim.x) {
      const long long t = e / M;
      const int m = (int)(e - t * M);
      cs[(base + t) * M + m] = sm[(off + t) * SUB_PAD + m];
    }
  }
}

// Downward, levels l0 .. L-1 of one subtree (target root r at level l0);
// writes the final leaf level.  blockIdx.x = vs * R + r.
template <bool NODAL>
__global__ void __launch_bounds__(32 * M) k_down_sub(double *c, Geo g, int l0, int d) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ double sm[];
  __shared__ double sB[tree_mat_size<NODAL>()];
  load_tree_mat<NODAL, false>(sB);
  const long long R = 4LL << l0;
  const long long vs = blockIdx.x / R, r = blockIdx.x - vs * R;
  double *cs = c + vs * g.slots * M;
  // level l0 + k of the subtree: 2^k nodes at sm + (2^k - 1) * SUB_PAD
  for (int k = 0; k <= d; k++) {
    const int nk = 1 << k;
    const int l = l0 + k;
    const long long nslot = (4LL << l) - 2, base = 2 * (long long)blocks_before((size_t)l);
    double *lev = sm + (nk - 1) * SUB_PAD;
    for (int e = threadIdx.x; e < nk * M; e += blockDim.x) {
      const int p = e / M, m = e - p * M;
      const long long t = r * nk + p;
      lev[p * SUB_PAD + m] = t < nslot ? cs[(base + t) * M + m] : 0.0;
    }
  }
  __syncthreads();
  for (int k = 0; k < d; k++) {
    const int nk = 1 << k;
    const long long nslot = (4LL << (l0 + k)) - 2;
    double *par = sm + (nk - 1) * SUB_PAD, *child = sm + (2 * nk - 1) * SUB_PAD;
    for (int it = threadIdx.x; it < nk * M; it += blockDim.x) {  // dense (node, row) items
      const int p = it & (nk - 1), i = it >> k;
      if (r * nk + p >= nslot) continue;
      double d0, d1;
      row_down<NODAL>(sB, par + p * SUB_PAD, i, d0, d1);
      child[(2 * p) * SUB_PAD + i] += d0;
      child[(2 * p + 1) * SUB_PAD + i] += d1;
    }
    __syncthreads();
  }
  const int nl = 1 << d;
  const double *leaf = sm + (nl - 1) * SUB_PAD;
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
    const int p = e / M, m = e - p * M;
    const long long t = r * nl + p;
    if (t < g.K) cs[(g.leaf_base + t) * M + m] = leaf[p * SUB_PAD + m];
  }
}

// Step 3: far-field blocks.  Ablk: the three 18x18 blocks of a block owning
// slots 2 gb, 2 gb + 1 of the tree ws / cs of one (vector, parity):
// c0 = A0 w0 + A1 w1, c1 = A2 w1 (leg2cheb.c:1419-1435).
__device__ __forceinline__ void far_item(const double *__restrict__ Ablk,
                                         const double *__restrict__ ws, double *__restrict__ cs,
                                         long long gb, int m) {
  const double *A0 = Ablk + m * M;
  const double *A1 = A0 + MM, *A2 = A1 + MM;
  const double *w0 = ws + 2 * gb * M, *w1 = w0 + M;
  double t0 = 0.0, t1 = 0.0, t2 = 0.0, u0 = 0.0, u1 = 0.0, u2 = 0.0;
#pragma unroll
  for (int k = 0; k < M; k += 2) {
    t0 = fma(A0[k], w0[k], t0);
    t1 = fma(A1[k], w1[k], t1);
    t2 = fma(A2[k], w1[k], t2);
    u0 = fma(A0[k + 1], w0[k + 1], u0);
    u1 = fma(A1[k + 1], w1[k + 1], u1);
    u2 = fma(A2[k + 1], w1[k + 1], u2);
  }
  double *c0 = cs + 2 * gb * M;
  c0[m] = (t0 + u0) + (t1 + u1);
  c0[M + m] = t2 + u2;
}

// Every level at once: block gb's A blocks start at 3 gb M^2.  A thread forms
// row m of block gb for both parities of its vector: its three A rows are read
// once, 16 bytes at a time (rows are 144 bytes, 16-byte aligned, as are the
// tree slots), and each parity's sums are accumulated in far_item's order.
__global__ void __launch_bounds__(256) k_far(const double *__restrict__ A,
                                             const double *__restrict__ w,
                                             double *__restrict__ c, Geo g, long long nblocks) {
  pdl_wait();
  pdl_trigger();
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long per_v = nblocks * M;
  if (idx >= g.count * per_v) return;
  const long long v = idx / per_v, rem = idx - v * per_v, gb = rem / M;
  const int m = (int)(rem - gb * M);
  const double2 *A0 = reinterpret_cast<const double2 *>(A + 3 * gb * MM + m * M);
  const double2 *A1 = A0 + MM / 2, *A2 = A1 + MM / 2;
  double t0[2] = {0.0, 0.0}, t1[2] = {0.0, 0.0}, t2[2] = {0.0, 0.0};
  double u0[2] = {0.0, 0.0}, u1[2] = {0.0, 0.0}, u2[2] = {0.0, 0.0};
#pragma unroll
  for (int k2 = 0; k2 < M / 2; k2++) {
    const double2 a0 = A0[k2], a1 = A1[k2], a2 = A2[k2];
#pragma unroll
    for (int sg = 0; sg < 2; sg++) {
      const double2 *ws = reinterpret_cast<const double2 *>(w + ((2 * v + sg) * g.slots + 2 * gb) * M);
      const double2 x0 = ws[k2], x1 = ws[M / 2 + k2];
      t0[sg] = fma(a0.x, x0.x, t0[sg]);
      t1[sg] = fma(a1.x, x1.x, t1[sg]);
      t2[sg] = fma(a2.x, x1.x, t2[sg]);
      u0[sg] = fma(a0.y, x0.y, u0[sg]);
      u1[sg] = fma(a1.y, x1.y, u1[sg]);
      u2[sg] = fma(a2.y, x1.y, u2[sg]);
    }
  }
#pragma unroll
  for (int sg = 0; sg < 2; sg++) {
    double *c0 = c + ((2 * v + sg) * g.slots + 2 * gb) * M;
    c0[m] = (t0[sg] + u0[sg]) + (t1[sg] + u1[sg]);
    c0[M + m] = t2[sg] + u2[sg];
  }
}

// Step 4, one level: parent target slot t of level l into children 2t, 2t+1 of
// level l+1 through the compact upper (transposed) binomial matrix: se/so sum the
// columns of equal/opposite parity to the row, child0 += se + so,
// child1 += se - so (leg2cheb.c:603-618).  Tiled as k_tree_up: the M parent
// coefficients of TREE_TILE parents staged in shared memory, warp i computes row i.
template <bool NODAL = false>
__device__ __forceinline__ void tree_down_tile(const double *const *par, double *const *child,
                                               const double *sB, double *sx) {
  for (int e = threadIdx.x; e < TREE_TILE * M; e += blockDim.x) {
    const int p = e / M, q = e - p * M;
    sx[p * TREE_PAD + q] = child[p] ? par[p][q] : 0.0;
  }
  __syncthreads();
  const int i = threadIdx.x >> 5, p = threadIdx.x & 31;
  if (i >= M || child[p] == nullptr) return;
  double d0, d1;
  row_down<NODAL>(sB, sx + p * TREE_PAD, i, d0, d1);
  double *ch = child[p];
  ch[i] += d0;
  ch[M + i] += d1;
}

template <bool NODAL>
__global__ void __launch_bounds__(32 * M) k_tree_down(double *c, Geo g, long long parent_base,
                                                      long long child_base, long long nparent) {
  pdl_wait();
  pdl_trigger();
  __shared__ double sB[tree_mat_size<NODAL>()];
  __shared__ double sx[TREE_TILE * TREE_PAD];
  __shared__ const double *par[TREE_TILE];
  __shared__ double *child[TREE_TILE];
  load_tree_mat<NODAL, false>(sB);
  if (threadIdx.x < TREE_TILE) {
    const long long item = (long long)blockIdx.x * TREE_TILE + threadIdx.x;
    const long long nitem = g.count * 2 * nparent;
    const long long vs = item / nparent, tp = item - vs * nparent;
    par[threadIdx.x] = c + (vs * g.slots + parent_base + tp) * M;
    child[threadIdx.x] = item < nitem ? c + (vs * g.slots + child_base + 2 * tp) * M : nullptr;
  }
  __syncthreads();
  tree_down_tile<NODAL>(par, child, sB, sx);
}

// Step 5 + scaling: out[j] = scale_j (y[j] + sum_m c[L-1][tau][m] T_sg[i][m]) with
// tau = j / h, sg = j & 1, i = (j - tau h)/2; no far field for tau >= K.
// L2C scale 2/pi (and 1/2 at j = 0, leg2cheb.c:360-374); C2L scale j + 1/2
// (leg2cheb.c:519-532).  cv: this vector's c; yv: its y; outv: its output line.
__device__ __forceinline__ void leaf_down_item(const double *__restrict__ cv,
                                               const double *__restrict__ T,
                                               const double *__restrict__ yv, double *outv,
                                               const Geo &g, int c2l, long long j) {
  const long long tau = j / g.h;
  double far = 0.0;
  if (tau < g.K) {
    const int sg = (int)(j & 1);
    const long long i = (j - tau * g.h) >> 1;
    const double *cc = cv + ((long long)sg * g.slots + g.leaf_base + tau) * M;
    const double *Ti = T + ((size_t)sg * g.s + i) * M;
    double f1 = 0.0;
#pragma unroll
    for (int m = 0; m < M; m += 2) {
      far = fma(cc[m], Ti[m], far);
      f1 = fma(cc[m + 1], Ti[m + 1], f1);
    }
    far += f1;
  }
  double val = yv[j] + far;
  if (!c2l) {
    val = val * l2c_out_scale(j);
  } else {
    val = val * dyadic(2 * (unsigned long long)j + 1, -1);  // j + 1/2
  }
  outv[j * g.stride] = val;
}

__global__ void __launch_bounds__(256) k_leaf_down(const double *__restrict__ c,
                                                   const double *__restrict__ T,
                                                   const double *__restrict__ y, double *out,
                                                   Geo g, int c2l) {
  pdl_wait();
  pdl_trigger();
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.count * g.N) return;
  const long long v = idx / g.N, j = idx - v * g.N;
  leaf_down_item(c + v * 2 * g.slots * M, T, y + v * g.N, out + v * g.dist, g, c2l, j);
}

// Direct O(N^2) transform for L < 1 (leg2cheb.c:152-234), with the reference's
// contract: out[0..N) is zeroed contiguously before the line is written, the
// L2C input is read contiguously, L2C accumulates into line elements past N.
// u, b: this vector's input and output line.
__device__ __forceinline__ void direct_item(const double *u, double *b,
                                            const double *__restrict__ a,
                                            const double *__restrict__ an,
                                            const double *__restrict__ dn, const Geo &g, int c2l,
                                            long long i) {
  double val;
  if (!c2l) {
    val = 0.0;
    for (long long k = 0; i + 2 * k < g.N; k++)
      val = fma((a[k] * TWO_OVER_PI) * a[k + i], u[i + 2 * k], val);
    if (i == 0) val = val / 2;
    if (i * g.stride >= g.N) val = b[i * g.stride] + val;
  } else {
    const double vi = (i == 0) ? u[0] : u[i * g.stride] * dyadic((unsigned long long)i, 0);
    val = (SQRT_PI * vi) * an[i];
    for (long long k = 1; i + 2 * k < g.N; k++) {
      const long long n = i + 2 * k;
      val = fma(-(dn[k] * an[k + i]), u[n * g.stride] * dyadic((unsigned long long)n, 0), val);
    }
    val = val * dyadic(2 * (unsigned long long)i + 1, -1);  // i + 1/2
  }
  if (g.stride > 1 && (i % g.stride) != 0) b[i] = 0.0;  // contiguous zeroing of [0, N)
  b[i * g.stride] = val;
}

__global__ void __launch_bounds__(256) k_direct(const double *in, double *out,
                                                const double *__restrict__ a,
                                                const double *__restrict__ an,
                                                const double *__restrict__ dn, Geo g, int c2l) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.count * g.N) return;
  const long long v = idx / g.N, i = idx - v * g.N;
  direct_item(in + v * g.dist, out + v * g.dist, a, an, dn, g, c2l, i);
}

inline unsigned blocks_for(long long n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

// ---------------------------------------------------------------------------
// Band of a batch as dense register tiles (batches of at least BT_MIN_COUNT
// vectors, leaf size s a multiple of 8 in [16, 64]; the band sums of directM /
// directL, leg2cheb.c:236-302 and :392-459).
//
// For a full block b < nL-1 and parity p the band is a small dense product
//   Y[i'][v] = sum_{m' = i' .. 2s-1} W'[m'][i'] X[m'][v],
// output j = b h + 2 i' + p, source x[v][b h + 2 m' + p], and the weight
// W'[m'][i'] = near_weight(k = m' - i', j) (the term k of output j).  A CTA of
// BT_WARPS warps owns a chunk of VCH = 32 C vectors and walks a run of
// consecutive blocks: block b reads the two half windows x[v][(b + e) h + [0, h)]
// (e = 0, 1), which pass through a ring of three shared-memory slots (rows of
// 2s + 1 doubles, odd, so the lanes of a warp hit distinct banks), each filled
// by cp.async one block ahead; at s = 16 the block's weights come the same way
// (two buffers), at larger s from L2.  Every lane owns C vectors; every warp
// owns row groups (4 consecutive rows i' of one parity) dealt in a snake order
// of their trip counts 2s - i'0, so the warps run equal numbers of FMAs.  A
// thread thus holds a 4 x C tile: per m' four weights (one address for the
// whole warp: a table entry or, without the table, the same products formed on
// the fly) and C shared-memory loads feed 4 C independent FMAs.  With this much
// independent work a few warps keep the FP64 pipe busy, so the kernel runs on
// one or two CTAs per SM and leaves the SM's other pipes, most of its
// registers and shared memory to the far-field chain beside it.  Each output
// sums its terms in order of k in one FMA chain from zero, then
// y = out_in + sum, staged through the slot the block no longer needs and
// written a row at a time.  The last (ragged) block takes k_near's sums, an
// output of 8 vectors per thread, as the first work units of the same launch.  The leaf
// size is a template parameter, so every loop bound and index below is a
// compile-time constant or a 32-bit offset.
// ---------------------------------------------------------------------------
constexpr int BT_WARPS = 4;
constexpr int BT_THREADS = 32 * BT_WARPS;
constexpr long long BT_MIN_COUNT = 64;

// CC: vectors per lane (the default, or 1 for the thin variant at s = 16,
// band_tile_thin).
template <int S, int CC = (S <= 32 ? 2 : 1)>
struct BandTile {
  static constexpr int H = 2 * S;
  static constexpr int C = CC;                // vectors per lane
  static constexpr int VCH = 32 * C;          // vectors per chunk
  static constexpr int LD = 2 * S + 1;        // slot row (odd)
  static constexpr int SLOT = VCH * LD;       // doubles per slot
  static constexpr int GROUPS = S / 2;        // row groups: 2 parities x s/4
  static constexpr int GPW = (GROUPS + BT_WARPS - 1) / BT_WARPS;
  // s = 16: each warp runs a pair of same-parity row groups (g, s/4 - 1 - g)
  // in one pass (band_tile_pair); larger leaves, whose groups have longer
  // loops, one group at a time (their registers would not hold a pair's sums)
  static constexpr bool PAIRED = S == 16;
  static constexpr int PAIRS = S / 4;
  static constexpr int PPW = (PAIRS + BT_WARPS - 1) / BT_WARPS;
  static constexpr int WB = 4 * S * S;        // weights of one block, both parities
  static constexpr bool WS = S == 16;         // weights staged in shared memory
  static constexpr size_t SMEM = (3 * (size_t)SLOT + (WS ? 2 * (size_t)WB : 0)) * sizeof(double);
};

// Vectors per lane of the tiled band (thin: the thin variant, s = 16 only).
__host__ __device__ inline int band_tile_c(long long s, bool thin = false) {
  return thin && s == 16 ? 1 : s <= 32 ? 2 : 1;
}
// Entries of the dense weight table: (nL - 1) blocks x 2 parities x 2s x s.
inline size_t band_tile_table_size(size_t N, size_t s) {
  const size_t h = 2 * s, nL = N / h;
  return nL >= 2 ? (nL - 1) * 4 * s * s : 0;
}

// Plan time: the dense table W'[b][p][m'][i'] (zero where m' < i').
__global__ void k_band_tile_weights(double *__restrict__ Wt, const double *__restrict__ a,
                                    const double *__restrict__ an,
                                    const double *__restrict__ dn, Geo g, int c2l) {
  const long long n = (g.nL - 1) * 4 * g.s * g.s;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const long long ip = idx % g.s, mp = (idx / g.s) % (2 * g.s), bp = idx / (2 * g.s * g.s);
  const long long b = bp >> 1, p = bp & 1;
  const long long j = b * g.h + 2 * ip + p;
  Wt[idx] = mp >= ip ? near_weight(c2l, mp - ip, j, a, an, dn) : 0.0;
}

// One term step m' of a row group: rows r < ROWS of the 4 (the others have no
// term at this m').  W (TAB): the four weights (16-byte aligned); without TAB
// they are formed here (output j0 + 2 r, term k = m' - i'0 - r).
template <int C, int ROWS, bool TAB>
__device__ __forceinline__ void band_tile_step(const double *__restrict__ xs, int ld,
                                               const double *W, int k0, long long j0, int c2l,
                                               const double *__restrict__ a,
                                               const double *__restrict__ an,
                                               const double *__restrict__ dn,
                                               double (&acc)[4][C]) {
  double w[4];
  if (TAB) {
    const double2 q0 = reinterpret_cast<const double2 *>(W)[0];
    const double2 q1 = reinterpret_cast<const double2 *>(W)[1];
    w[0] = q0.x;
    w[1] = q0.y;
    w[2] = q1.x;
    w[3] = q1.y;
  } else {
#pragma unroll
    for (int r = 0; r < 4; r++)
      w[r] = r < ROWS ? near_weight(c2l, k0 - r, j0 + 2 * r, a, an, dn) : 0.0;
  }
  double xv[C];
#pragma unroll
  for (int c = 0; c < C; c++) xv[c] = xs[c * 32 * ld];
#pragma unroll
  for (int r = 0; r < ROWS; r++)
#pragma unroll
    for (int c = 0; c < C; c++) acc[r][c] = fma(w[r], xv[c], acc[r][c]);
}

// Row group (parity p, rows i'0 .. i'0 + 3) of one block for the lane's C
// vectors.  sA / sB: the lane's rows in the two half-window slots; Wg: the
// group's weights at m' = 0 (row stride S), or nullptr.
template <int S, int CC, bool TAB>
__device__ __forceinline__ void band_tile_group(const double *__restrict__ sA,
                                                const double *__restrict__ sB,
                                                const double *Wg, int p, int ip0, long long j0,
                                                int c2l, const double *__restrict__ a,
                                                const double *__restrict__ an,
                                                const double *__restrict__ dn,
                                                double (&acc)[4][CC]) {
  using BT = BandTile<S, CC>;
  constexpr int C = BT::C, LD = BT::LD;
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < C; c++) acc[r][c] = 0.0;
  // m' = i'0 .. i'0 + 2: only rows r <= m' - i'0 have a term (i'0 + 3 < s)
  band_tile_step<C, 1, TAB>(sA + 2 * ip0 + p, LD, TAB ? Wg + ip0 * S : nullptr, 0, j0, c2l, a,
                            an, dn, acc);
  band_tile_step<C, 2, TAB>(sA + 2 * ip0 + 2 + p, LD, TAB ? Wg + (ip0 + 1) * S : nullptr, 1, j0,
                            c2l, a, an, dn, acc);
  band_tile_step<C, 3, TAB>(sA + 2 * ip0 + 4 + p, LD, TAB ? Wg + (ip0 + 2) * S : nullptr, 2, j0,
                            c2l, a, an, dn, acc);
#pragma unroll 4
  for (int mp = ip0 + 3; mp < S; mp++)
    band_tile_step<C, 4, TAB>(sA + 2 * mp + p, LD, TAB ? Wg + mp * S : nullptr, mp - ip0, j0,
                              c2l, a, an, dn, acc);
#pragma unroll(S <= 16 ? S : 8)
  for (int mp = S; mp < 2 * S; mp++)
    band_tile_step<C, 4, TAB>(sB + 2 * (mp - S) + p, LD, TAB ? Wg + mp * S : nullptr, mp - ip0,
                              j0, c2l, a, an, dn, acc);
}

// One term step m' of two row groups of one parity: group a (all 4 rows) and
// group b (rows r < ROWS_B): they read the same source x, so a step issues
// 4 C + ROWS_B C independent FMAs from two weight quads and C shared loads.
template <int C, int ROWS_B, bool TAB>
__device__ __forceinline__ void band_tile_step2(const double *__restrict__ xs, int ld,
                                                const double *Wa, const double *Wb, int ka0,
                                                int kb0, long long ja0, long long jb0, int c2l,
                                                const double *__restrict__ a,
                                                const double *__restrict__ an,
                                                const double *__restrict__ dn,
                                                double (&acca)[4][C], double (&accb)[4][C]) {
  double wa[4], wb[4];
  if (TAB) {
    const double2 a0 = reinterpret_cast<const double2 *>(Wa)[0];
    const double2 a1 = reinterpret_cast<const double2 *>(Wa)[1];
    const double2 b0 = reinterpret_cast<const double2 *>(Wb)[0];
    const double2 b1 = reinterpret_cast<const double2 *>(Wb)[1];
    wa[0] = a0.x;
    wa[1] = a0.y;
    wa[2] = a1.x;
    wa[3] = a1.y;
    wb[0] = b0.x;
    wb[1] = b0.y;
    wb[2] = b1.x;
    wb[3] = b1.y;
  } else {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      wa[r] = near_weight(c2l, ka0 - r, ja0 + 2 * r, a, an, dn);
      wb[r] = r < ROWS_B ? near_weight(c2l, kb0 - r, jb0 + 2 * r, a, an, dn) : 0.0;
    }
  }
  double xv[C];
#pragma unroll
  for (int c = 0; c < C; c++) xv[c] = xs[c * 32 * ld];
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < C; c++) acca[r][c] = fma(wa[r], xv[c], acca[r][c]);
#pragma unroll
  for (int r = 0; r < ROWS_B; r++)
#pragma unroll
    for (int c = 0; c < C; c++) accb[r][c] = fma(wb[r], xv[c], accb[r][c]);
}

// Two row groups of one parity in one pass: a from row ia, b from row ib
// (ia + 4 <= ib <= s - 4).  Group a runs alone over m' = ia .. ib-1; from
// m' = ib both share each source, which doubles the independent FMAs per step
// (more work per warp between loads, so fewer warps keep the FP64 pipe busy).
// Each row's terms are still summed in order of k in one chain.
template <int S, int CC, bool TAB>
__device__ __forceinline__ void band_tile_pair(const double *__restrict__ sA,
                                               const double *__restrict__ sB, const double *Wga,
                                               const double *Wgb, int p, int ia, int ib,
                                               long long ja0, long long jb0, int c2l,
                                               const double *__restrict__ a,
                                               const double *__restrict__ an,
                                               const double *__restrict__ dn,
                                               double (&acca)[4][CC], double (&accb)[4][CC]) {
  using BT = BandTile<S, CC>;
  constexpr int C = BT::C, LD = BT::LD;
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < C; c++) acca[r][c] = accb[r][c] = 0.0;
  // group a alone: its first three steps have rows r <= m' - ia only
  band_tile_step<C, 1, TAB>(sA + 2 * ia + p, LD, TAB ? Wga + ia * S : nullptr, 0, ja0, c2l, a,
                            an, dn, acca);
  band_tile_step<C, 2, TAB>(sA + 2 * ia + 2 + p, LD, TAB ? Wga + (ia + 1) * S : nullptr, 1, ja0,
                            c2l, a, an, dn, acca);
  band_tile_step<C, 3, TAB>(sA + 2 * ia + 4 + p, LD, TAB ? Wga + (ia + 2) * S : nullptr, 2, ja0,
                            c2l, a, an, dn, acca);
#pragma unroll 4
  for (int mp = ia + 3; mp < ib; mp++)
    band_tile_step<C, 4, TAB>(sA + 2 * mp + p, LD, TAB ? Wga + mp * S : nullptr, mp - ia, ja0,
                              c2l, a, an, dn, acca);
  // both groups (b's first three steps with rows r <= m' - ib); ib + 2 < s
  band_tile_step2<C, 1, TAB>(sA + 2 * ib + p, LD, TAB ? Wga + ib * S : nullptr,
                             TAB ? Wgb + ib * S : nullptr, ib - ia, 0, ja0, jb0, c2l, a, an, dn,
                             acca, accb);
  band_tile_step2<C, 2, TAB>(sA + 2 * ib + 2 + p, LD, TAB ? Wga + (ib + 1) * S : nullptr,
                             TAB ? Wgb + (ib + 1) * S : nullptr, ib + 1 - ia, 1, ja0, jb0, c2l, a,
                             an, dn, acca, accb);
  band_tile_step2<C, 3, TAB>(sA + 2 * ib + 4 + p, LD, TAB ? Wga + (ib + 2) * S : nullptr,
                             TAB ? Wgb + (ib + 2) * S : nullptr, ib + 2 - ia, 2, ja0, jb0, c2l, a,
                             an, dn, acca, accb);
#pragma unroll 4
  for (int mp = ib + 3; mp < S; mp++)
    band_tile_step2<C, 4, TAB>(sA + 2 * mp + p, LD, TAB ? Wga + mp * S : nullptr,
                               TAB ? Wgb + mp * S : nullptr, mp - ia, mp - ib, ja0, jb0, c2l, a,
                               an, dn, acca, accb);
#pragma unroll(S <= 16 ? S : 8)
  for (int mp = S; mp < 2 * S; mp++)
    band_tile_step2<C, 4, TAB>(sB + 2 * (mp - S) + p, LD, TAB ? Wga + mp * S : nullptr,
                               TAB ? Wgb + mp * S : nullptr, mp - ia, mp - ib, ja0, jb0, c2l, a,
                               an, dn, acca, accb);
}

// Copies of half window hw of the chunk's vectors into slot dst (zeros for
// vectors past the batch).
template <int S, int CC>
__device__ __forceinline__ void band_tile_fill(double *dst, const double *__restrict__ x,
                                               const Geo &g, long long v0, long long hw) {
  using BT = BandTile<S, CC>;
#pragma unroll 4
  for (int idx = threadIdx.x; idx < BT::VCH * BT::H; idx += BT_THREADS) {
    const int vl = idx / BT::H, m = idx % BT::H;
    const long long v = v0 + vl;
    const bool live = v < g.count;
    l2c_oz::cp_async8(dst + vl * BT::LD + m, live ? x + v * g.N + hw * BT::H + m : x,
                      live ? 8 : 0);
  }
}
// Copies of the weights of block wb into wdst.
template <int S>
__device__ __forceinline__ void band_tile_fill_w(double *wdst, const double *__restrict__ Wt,
                                                 long long wb) {
  using BT = BandTile<S>;
  const double *src = Wt + wb * BT::WB;
#pragma unroll
  for (int idx = threadIdx.x; idx < BT::WB / 2; idx += BT_THREADS)
    l2c_oz::cp_async16(wdst + 2 * idx, src + 2 * idx, 16);
}

// Work units: first, per vector chunk, its last (ragged) block; then unit
// nchunk + u: vector chunk u % nchunk, blocks [seg bseg, (seg + 1) bseg) of
// the nL - 1 full ones, seg = u / nchunk (a segment's chunks run side by side,
// so its weights are read from L2 by all of them).  Warp w takes the row
// groups q = 8 t' + w and 8 t' + 7 - w (t' = 0, 1, ...), q < s/2.  At most
// 128 registers per thread, so that one or two of these CTAs leave most of an
// SM's register file to the kernels beside them (the thin variant, one vector
// per lane: at most 64, and half the shared memory).
template <int S, bool TAB, int CC = BandTile<S>::C>
__global__ void __launch_bounds__(BT_THREADS, CC < BandTile<S>::C ? 8 : 4)
    k_band_tile(const double *__restrict__ x, const double *out, double *__restrict__ y,
                const double *__restrict__ Wt, const double *__restrict__ a,
                const double *__restrict__ an, const double *__restrict__ dn, Geo g, int c2l,
                long long nchunk, long long bseg) {
  using BT = BandTile<S, CC>;
  constexpr int C = BT::C, VCH = BT::VCH, LD = BT::LD, H = BT::H;
  constexpr bool WS = TAB && BT::WS;
  extern __shared__ __align__(16) double bt_smem[];
  double *wsm = bt_smem + 3 * BT::SLOT;  // two weight buffers (WS)
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long nfull = g.nL - 1, nseg = (nfull + bseg - 1) / bseg;
  const long long jlast = nfull * H, ntail = g.N - jlast;
  for (long long u = blockIdx.x; u < nchunk * (nseg + 1); u += gridDim.x) {
    if (u < nchunk) {
      // the last (ragged) block of chunk u: k_near's sums (weights formed on
      // the fly, each shared by TV vectors; the same bits as k_near), an
      // output of TV vectors per thread (4 in the thin variant, within its
      // registers), a vector at a time past the last full group
      constexpr int TV = CC < BandTile<S>::C ? 4 : 8;  // vectors per thread
      const long long vb = u * VCH, nv = g.count - vb < VCH ? g.count - vb : VCH;
      const long long ngrp = nv / TV;
      for (long long idx = threadIdx.x; idx < (ngrp + (nv - TV * ngrp)) * ntail;
           idx += BT_THREADS) {
        const long long grp = idx / ntail, j = jlast + idx % ntail;
        if (grp < ngrp) {
          const long long v0 = vb + TV * grp;
          double res[TV];
          near_sums<TV>(x + v0 * g.N + j, g.N, a, an, dn, nullptr, g, c2l, j, res);
#pragma unroll
          for (int e = 0; e < TV; e++)
            y[(v0 + e) * g.N + j] = out[(v0 + e) * g.dist + j * g.stride] + res[e];
        } else {
          const long long v = vb + TV * ngrp + (grp - ngrp);
          double res[1];
          near_sums<1>(x + v * g.N + j, g.N, a, an, dn, nullptr, g, c2l, j, res);
          y[v * g.N + j] = out[v * g.dist + j * g.stride] + res[0];
        }
      }
      continue;
    }
    const long long uu = u - nchunk;
    const long long v0 = (uu % nchunk) * VCH, seg = uu / nchunk;
    const long long b0 = seg * bseg, b1 = b0 + bseg < nfull ? b0 + bseg : nfull;
    // half windows b0 and b0 + 1 (block b0 needs both), block b0's weights
    band_tile_fill<S, CC>(bt_smem + (int)(b0 % 3) * BT::SLOT, x, g, v0, b0);
    if (WS) band_tile_fill_w<S>(wsm + (int)(b0 & 1) * BT::WB, Wt, b0);
    l2c_oz::cp_commit();
    band_tile_fill<S, CC>(bt_smem + (int)((b0 + 1) % 3) * BT::SLOT, x, g, v0, b0 + 1);
    l2c_oz::cp_commit();
    for (long long b = b0; b < b1; b++) {
      // half window b + 2 and block b + 1's weights, one block ahead
      if (b + 2 <= b1) {
        band_tile_fill<S, CC>(bt_smem + (int)((b + 2) % 3) * BT::SLOT, x, g, v0, b + 2);
        if (WS) band_tile_fill_w<S>(wsm + (int)((b + 1) & 1) * BT::WB, Wt, b + 1);
      }
      l2c_oz::cp_commit();
      l2c_oz::cp_wait1();  // halves b, b + 1 and block b's weights have landed
      __syncthreads();
      double *sA = bt_smem + (int)(b % 3) * BT::SLOT;
      const double *sB = bt_smem + (int)((b + 1) % 3) * BT::SLOT;
      const double *Wb = !TAB ? nullptr : WS ? wsm + (int)(b & 1) * BT::WB : Wt + b * BT::WB;
      if constexpr (BT::PAIRED) {
        // warp w: pairs q = w, w + 4, ... of same-parity row groups (g, s/4-1-g)
        double res[BT::PPW][2][4][C];
  #pragma unroll
        for (int t = 0; t < BT::PPW; t++) {
          const int q = warp + BT_WARPS * t;
          if (q < BT::PAIRS) {
            const int p = q / (S / 8), ga = q % (S / 8), ia = 4 * ga, ib = S - 4 - ia;
            const double *Wp = TAB ? Wb + p * 2 * S * S : nullptr;
            band_tile_pair<S, CC, TAB>(sA + lane * LD, sB + lane * LD, TAB ? Wp + ia : nullptr,
                                       TAB ? Wp + ib : nullptr, p, ia, ib, b * H + 2 * ia + p,
                                       b * H + 2 * ib + p, c2l, a, an, dn, res[t][0],
                                       res[t][1]);
          }
        }
        __syncthreads();  // every warp is done reading slots A and B
        // the sums, staged in slot A (its inputs are no longer needed)
  #pragma unroll
        for (int t = 0; t < BT::PPW; t++) {
          const int q = warp + BT_WARPS * t;
          if (q < BT::PAIRS) {
            const int p = q / (S / 8), ia = 4 * (q % (S / 8)), ib = S - 4 - ia;
  #pragma unroll
            for (int r = 0; r < 4; r++)
  #pragma unroll
              for (int c = 0; c < C; c++) {
                sA[(lane + 32 * c) * LD + 2 * (ia + r) + p] = res[t][0][r][c];
                sA[(lane + 32 * c) * LD + 2 * (ib + r) + p] = res[t][1][r][c];
              }
          }
        }
      } else {
        double res[BT::GPW][4][C];
  #pragma unroll
        for (int t = 0; t < BT::GPW; t++) {
          const int q = 8 * (t >> 1) + ((t & 1) ? 2 * BT_WARPS - 1 - warp : warp);
          if (q < BT::GROUPS) {
            const int p = q & 1, ip0 = 4 * (q >> 1);
            band_tile_group<S, CC, TAB>(sA + lane * LD, sB + lane * LD,
                                        TAB ? Wb + p * 2 * S * S + ip0 : nullptr, p, ip0,
                                        b * H + 2 * ip0 + p, c2l, a, an, dn, res[t]);
          }
        }
        __syncthreads();  // every warp is done reading slots A and B
        // the sums, staged in slot A (its inputs are no longer needed)
  #pragma unroll
        for (int t = 0; t < BT::GPW; t++) {
          const int q = 8 * (t >> 1) + ((t & 1) ? 2 * BT_WARPS - 1 - warp : warp);
          if (q < BT::GROUPS)
  #pragma unroll
            for (int r = 0; r < 4; r++)
  #pragma unroll
              for (int c = 0; c < C; c++)
                sA[(lane + 32 * c) * LD + 2 * (4 * (q >> 1) + r) + (q & 1)] = res[t][r][c];
        }
      }
      __syncthreads();
      // y = out_in + band, a row of h outputs per vector (eight loads of the
      // thread in flight at a time)
#pragma unroll 8
      for (int idx = threadIdx.x; idx < VCH * H; idx += BT_THREADS) {
        const int vl = idx / H, i = idx % H;
        const long long v = v0 + vl;
        if (v < g.count) {
          const long long j = b * H + i;
          y[v * g.N + j] = out[v * g.dist + j * g.stride] + sA[vl * LD + i];
        }
      }
      __syncthreads();  // slot A is refilled next
    }
    l2c_oz::cp_wait0();
    __syncthreads();
  }
}

// Whether a batch's band takes k_band_tile: count >= BT_MIN_COUNT, s a
// multiple of 8 in [16, 64], at least one full block.
inline bool band_tile_ok(long long s, long long nL, long long count) {
  return count >= BT_MIN_COUNT && s % 8 == 0 && s >= 16 && s <= 64 && nL >= 2;
}

template <bool TAB>
using band_tile_fn = void (*)(const double *, const double *, double *, const double *,
                              const double *, const double *, const double *, Geo, int,
                              long long, long long);

template <bool TAB>
band_tile_fn<TAB> band_tile_kernel(long long s, bool thin = false) {
  switch (s / 8) {
    case 2: return thin ? k_band_tile<16, TAB, 1> : k_band_tile<16, TAB>;
    case 3: return k_band_tile<24, TAB>;
    case 4: return k_band_tile<32, TAB>;
    case 5: return k_band_tile<40, TAB>;
    case 6: return k_band_tile<48, TAB>;
    case 7: return k_band_tile<56, TAB>;
    default: return k_band_tile<64, TAB>;
  }
}

inline size_t band_tile_smem(long long s, bool thin = false) {
  switch (s / 8) {
    case 2: return thin ? BandTile<16, 1>::SMEM : BandTile<16>::SMEM;
    case 3: return BandTile<24>::SMEM;
    case 4: return BandTile<32>::SMEM;
    case 5: return BandTile<40>::SMEM;
    case 6: return BandTile<48>::SMEM;
    case 7: return BandTile<56>::SMEM;
    default: return BandTile<64>::SMEM;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Mixed-precision far field (L2C_PLAN_MIXED): the leaf, transfer and far-field
// products on FP16 tensor cores through l2c_ozaki.cuh, FP64-accurate with no
// FP64 instruction in the products; the near-field band, the final
// accumulation and scaling stay in FP64.  Every kernel: one warp per tile of
// 16 right-hand-side columns against a constant factor pre-sliced at plan time
// into per-lane fragments (l2c_oz::frag_index) that the CTA copies to shared
// memory once; each warp streams its tiles through a two-deep cp.async
// pipeline (the next tile's copies are in flight while one is computed).
// Between the products the moments w and c stay in the column format of
// l2c_oz::stage_cols (integers and one exponent per 18-coefficient column).
// ---------------------------------------------------------------------------
constexpr int MXW = 4;              // warps per CTA
constexpr int OZ_NT = 3;            // 18 outputs = 3 n-tiles of 8
constexpr int OZ_ROWS = 8 * OZ_NT;  // padded output rows
constexpr int OZ_META = 32;         // per-matrix ints: row shifts [0, 24), exponent offset [24]
constexpr int OZ_TLD = 42;          // staged row of 36 (K = 2M) values, padded
constexpr int OZ_CLD = 26;          // staged row of 18 (K = M) values, padded
__host__ __device__ constexpr int oz_words(int NT, int KC) { return l2c_oz::SLICES * NT * KC * 32; }

// Plan time: the fragment words and row exponent of one row n of a matrix with
// K columns (row(k) gives P[n][k]; rows past the matrix are zero).
template <class Row>
__host__ __device__ void oz_pack_row(Row row, bool live, int n, int K, int NT, int KC,
                                     unsigned *frag, int *E) {
  int e = l2c_oz::EXP_ZERO;
  if (live)
    for (int k = 0; k < K; k++) {
      const int ek = l2c_oz::exp_bound(row(k));
      e = e > ek ? e : ek;
    }
  E[n] = e;
  const int nt = n >> 3, g = n & 7;
  for (int c = 0; c < KC; c++)
    for (int t = 0; t < 4; t++) {
      const int k0 = 8 * c + 2 * t;
      const long long y0 = live && k0 < K ? l2c_oz::fixbal(row(k0), e) : l2c_oz::RBAL;
      const long long y1 = live && k0 + 1 < K ? l2c_oz::fixbal(row(k0 + 1), e) : l2c_oz::RBAL;
      for (int q = 1; q <= l2c_oz::SLICES; q++)
        frag[l2c_oz::frag_index(q, nt, c, 4 * g + t, NT, KC)] =
            l2c_oz::half_bits((int)l2c_oz::digit_f(y0, q)) |
            (l2c_oz::half_bits((int)l2c_oz::digit_f(y1, q)) << 16);
    }
}

// Producer metadata of a matrix with row exponents E[0, M): for a column with
// exponent Ec (entries below 2^Ec) and K <= 64 terms, output n is below
// K 2^(E[n] + Ec) <= 2^(Ec + Emax + 6); its integer T (value T 2^(Ec + E[n] - 52))
// is stored as T 2^(E[n] - Emax + 3) under the column exponent Ec + Emax + 7,
// so |V| < 2^61.  meta[n] = E[n] - Emax + 3, meta[24] = Emax + 7.
__host__ __device__ inline void oz_meta(const int *E, int *meta) {
  int emax = l2c_oz::EXP_ZERO;
  for (int n = 0; n < M; n++) emax = E[n] > emax ? E[n] : emax;
  for (int n = 0; n < OZ_META; n++) meta[n] = 0;
  for (int n = 0; n < M; n++) {
    const int sft = E[n] - emax + 3;
    meta[n] = sft < -63 ? -63 : sft;
  }
  meta[OZ_ROWS] = emax + 7;
}

// Far-field block fragments: block gb as one 40 x 40 matrix
//   [[A0 A1]   rows 0 .. 17: the block's first slot (slot 2 gb)
//    [ 0 A2]]  rows 18 .. 35: its second slot (2 gb + 1); rows 36 .. 39 zero
// over the two slots' 36 moments (columns 36 .. 39 zero), NT = 5 n-tiles and
// KC = 5 chunks: one product per data tile serves both output slots from one
// digit extraction.  Words at F + gb * OZ_FAR_WORDS, metadata at
// Pm + gb * 2 * OZ_META (part 0: rows 0 .. 17, part 1: rows 18 .. 35).  One
// thread per (block, part).
constexpr int OZ_FAR_NT = 5, OZ_FAR_KC = 5;
constexpr int OZ_FAR_WORDS = oz_words(OZ_FAR_NT, OZ_FAR_KC);
__global__ void k_oz_pack_far(const double *__restrict__ A, long long nblocks, unsigned *F,
                              int *Pm) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= nblocks * 2) return;
  const long long gb = idx >> 1;
  const int part = (int)(idx & 1);
  unsigned *Fb = F + gb * OZ_FAR_WORDS;
  int E[8 * OZ_FAR_NT];
  const int n0 = part ? M : 0, n1 = part ? 8 * OZ_FAR_NT : M;
  for (int n = n0; n < n1; n++) {
    const int r = n - n0;  // row of the part's blocks
    const double *Ar = A + 3 * gb * MM + (r < M ? r : 0) * M;
    if (part == 0)
      oz_pack_row([&](int k) { return k < M ? Ar[k] : Ar[MM + k - M]; }, true, n, 2 * M,
                  OZ_FAR_NT, OZ_FAR_KC, Fb, E);
    else
      oz_pack_row([&](int k) { return k < M ? 0.0 : Ar[2 * MM + k - M]; }, r < M, n, 2 * M,
                  OZ_FAR_NT, OZ_FAR_KC, Fb, E);
  }
  oz_meta(E + n0, Pm + (gb * 2 + part) * OZ_META);
}

// Copy nwords fragment words (and nint metadata ints) into shared memory.
__device__ __forceinline__ void oz_load_frag(unsigned *dst, const unsigned *__restrict__ src,
                                             int nwords, int *idst, const int *__restrict__ isrc,
                                             int nint) {
  const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
  uint4 *d4 = reinterpret_cast<uint4 *>(dst);
  for (int i = threadIdx.x; i < nwords / 4; i += blockDim.x) d4[i] = s4[i];
  for (int i = threadIdx.x; i < nint; i += blockDim.x) idst[i] = isrc[i];
}

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes));
}

// Per-warp pipeline over tiles first, first + step, ... < ntile: issue(tile,
// buf) starts the copies of a tile into buffer buf, work(tile, buf) computes it
// once they have landed.  NBUF = 2 copies the next tile during the current
// one; NBUF = 1 (half the shared memory per warp, so more warps per SM) waits
// for each tile's copies.
template <int NBUF = 2, class Issue, class Work>
__device__ __forceinline__ void oz_tile_loop(long long first, long long step, long long ntile,
                                             Issue issue, Work work) {
  if (first >= ntile) return;
  if constexpr (NBUF == 1) {
    for (long long tile = first; tile < ntile; tile += step) {
      issue(tile, 0);
      l2c_oz::cp_commit();
      l2c_oz::cp_wait0();
      __syncwarp();
      work(tile, 0);
      __syncwarp();
    }
    return;
  }
  issue(first, 0);
  l2c_oz::cp_commit();
  int buf = 0;
  for (long long tile = first; tile < ntile; tile += step) {
    if (tile + step < ntile) issue(tile + step, buf ^ 1);
    l2c_oz::cp_commit();
    l2c_oz::cp_wait1();
    __syncwarp();
    work(tile, buf);
    __syncwarp();
    buf ^= 1;
  }
}

// Combined integers of a 16 x (NT*8) tile; K past KMAX is split into two exact
// accumulations whose integers are added.  The split falls on a chunk pair
// (chunks 0-3, then 4..KC-1): fragment words are interleaved in pairs of
// chunks, each pair one 8-byte load.
template <int NT, int KC, int QMAX = l2c_oz::SLICES>
__device__ __forceinline__ void oz_tile_T(const unsigned *Pf, const long long *Ys, int yld, int ks,
                                          long long (&T)[NT][4]) {
  float acc[l2c_oz::NDIAG][NT][4];
  if constexpr (KC <= l2c_oz::KMAX / 8) {
    l2c_oz::mma_tile<NT, KC, 0, KC, QMAX>(Pf, Ys, yld, ks, acc);
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) T[nt][e] = l2c_oz::combine(acc, nt, e);
  } else {
    constexpr int CM = 4;
    static_assert(KC - CM <= l2c_oz::KMAX / 8, "two exact accumulations cover at most 10 chunks");
    l2c_oz::mma_tile<NT, KC, 0, CM, QMAX>(Pf, Ys, yld, ks, acc);
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) T[nt][e] = l2c_oz::combine(acc, nt, e);
    l2c_oz::mma_tile<NT, KC, CM, KC, QMAX>(Pf, Ys, yld, ks, acc);
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) T[nt][e] += l2c_oz::combine(acc, nt, e);
  }
}

// Producer epilogue of a 16 x 24 tile with 18 real output rows: the lane's
// 9 real outputs are n-tiles 0 and 1 (rows g, g+8; outputs 8nt + 2t, +1) and
// one element of n-tile 2, whose four real elements all sit in the quad's
// lane t = 0 and are dealt out one per lane.  put2(r, n, V0, V1) stores
// outputs n, n+1 of tile row r, put1(r, n, V) one output; rs[n] is the
// metadata row shift.
template <class Put2, class Put1>
__device__ __forceinline__ void oz_put18(const long long (&T)[OZ_NT][4], const int *rs, Put2 put2,
                                         Put1 put1) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 2; nt++)
#pragma unroll
    for (int hr = 0; hr < 2; hr++) {
      const int n = 8 * nt + 2 * t4;
      put2(g + 8 * hr, n, l2c_oz::shift_s64(T[nt][2 * hr], rs[n]),
           l2c_oz::shift_s64(T[nt][2 * hr + 1], rs[n + 1]));
    }
  const int src = lane & ~3;
  const long long v1 = __shfl_sync(0xffffffffu, T[2][1], src);
  const long long v2 = __shfl_sync(0xffffffffu, T[2][2], src);
  const long long v3 = __shfl_sync(0xffffffffu, T[2][3], src);
  const long long t9 = t4 == 0 ? T[2][0] : t4 == 1 ? v1 : t4 == 2 ? v2 : v3;
  const int n9 = 16 + (t4 & 1);
  put1(g + 8 * (t4 >> 1), n9, l2c_oz::shift_s64(t9, rs[n9]));
}

// oz_put18 for one n-tile at a time (T4: that n-tile's four integers), for
// products computed n-tile by n-tile (mma_nt).
template <class Put2, class Put1>
__device__ __forceinline__ void oz_put_nt(int nt, const long long (&T4)[4], const int *rs,
                                          Put2 put2, Put1 put1) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t4 = lane & 3;
  if (nt < 2) {
#pragma unroll
    for (int hr = 0; hr < 2; hr++) {
      const int n = 8 * nt + 2 * t4;
      put2(g + 8 * hr, n, l2c_oz::shift_s64(T4[2 * hr], rs[n]),
           l2c_oz::shift_s64(T4[2 * hr + 1], rs[n + 1]));
    }
    return;
  }
  const int src = lane & ~3;
  const long long v1 = __shfl_sync(0xffffffffu, T4[1], src);
  const long long v2 = __shfl_sync(0xffffffffu, T4[2], src);
  const long long v3 = __shfl_sync(0xffffffffu, T4[3], src);
  const long long t9 = t4 == 0 ? T4[0] : t4 == 1 ? v1 : t4 == 2 ? v2 : v3;
  const int n9 = 16 + (t4 & 1);
  put1(g + 8 * (t4 >> 1), n9, l2c_oz::shift_s64(t9, rs[n9]));
}

// Leaf up (step 1): tile = 16 consecutive leaf nodes of one vector; both
// parities from one staged stretch of x (node r's h inputs in row r, parity
// sg at even/odd positions).  P_sg = T_sg^T (18 x s), KC = ceil(s / 8).
// Single-buffered kernels (NBUF = 1) are held to 128 registers (four CTAs per
// SM) so the warps freed from the second buffer can be resident.
constexpr int oz_min_ctas(int NBUF) { return NBUF == 1 ? 4 : 1; }

template <int KC, int NBUF>
__global__ void __launch_bounds__(32 * MXW, oz_min_ctas(NBUF))
    k_mz_leaf_up(const double *__restrict__ x, long long *__restrict__ w, int *__restrict__ wE,
                 const unsigned *__restrict__ Pf, const int *__restrict__ Pm, Geo g,
                 int *__restrict__ bad) {
  constexpr int XLD = 16 * KC + 1, NW = oz_words(OZ_NT, KC);
  extern __shared__ __align__(16) unsigned char mz_smem[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
  unsigned *sP = reinterpret_cast<unsigned *>(mz_smem);
  int *sM = reinterpret_cast<int *>(sP + 2 * NW);
  int *Es = sM + 2 * OZ_META + wid * 32;
  double *Xw = reinterpret_cast<double *>(sM + 2 * OZ_META + 32 * MXW) + wid * NBUF * 16 * XLD;
  oz_load_frag(sP, Pf, 2 * NW, sM, Pm, 2 * OZ_META);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  const long long tpv = (g.K + 15) / 16, ntile = g.count * tpv;
  auto issue = [&](long long tile, int buf) {
    const long long v = tile / tpv, node0 = (tile - v * tpv) * 16;
    const double *xv = x + v * g.N;
    double *X = Xw + buf * 16 * XLD;
    for (int r = 0; r < 16; r++) {
      const long long base = (node0 + r + 2) * g.h;
      const bool live = node0 + r < g.K;
      for (int j = lane; j < g.h; j += 32) {
        const bool ok = live && base + j < g.N;
        l2c_oz::cp_async8(X + r * XLD + j, ok ? xv + base + j : xv, ok ? 8 : 0);
      }
    }
  };
  auto work = [&](long long tile, int buf) {
    const long long v = tile / tpv, node0 = (tile - v * tpv) * 16;
    double *X = Xw + buf * 16 * XLD;
    l2c_oz::stage_fix<8 * KC>(X, XLD, 2, (int)g.s, Es);
    l2c_oz::stage_fix<8 * KC>(X + 1, XLD, 2, (int)g.s, Es + 16);
    const long long *Ys = reinterpret_cast<const long long *>(X);
#pragma unroll 1
    for (int sg = 0; sg < 2; sg++) {
      const int *meta = sM + sg * OZ_META;
      long long *wcol = w + ((v * 2 + sg) * g.slots + g.leaf_base + node0) * M;
      const long long nrow = g.K - node0;
      auto put2 = [&](int r, int n, long long a, long long b) {
        if (r < nrow) *reinterpret_cast<longlong2 *>(wcol + r * M + n) = make_longlong2(a, b);
      };
      auto put1 = [&](int r, int n, long long a) {
        if (r < nrow) wcol[r * M + n] = a;
      };
      if constexpr (KC <= 3) {
        // one n-tile at a time from cached digits (fewer live accumulators)
        l2c_oz::Digits<KC> D;
        l2c_oz::load_digits<KC>(Ys + sg, XLD, 2, D);
#pragma unroll
        for (int nt = 0; nt < OZ_NT; nt++) {
          float acc[l2c_oz::NDIAG][4];
          l2c_oz::mma_nt<OZ_NT, KC>(sP + sg * NW, D, nt, acc);
          long long T4[4];
#pragma unroll
          for (int e = 0; e < 4; e++) T4[e] = l2c_oz::combine1(acc, e);
          oz_put_nt(nt, T4, meta, put2, put1);
        }
      } else {
        long long T[OZ_NT][4];
        oz_tile_T<OZ_NT, KC>(sP + sg * NW, Ys + sg, XLD, 2, T);
        oz_put18(T, meta, put2, put1);
      }
      if (t4 == 0)
        for (int hr = 0; hr < 2; hr++) {
          const int r = gq + 8 * hr;
          if (r < nrow) {
            wE[(v * 2 + sg) * g.slots + g.leaf_base + node0 + r] = Es[sg * 16 + r] + meta[OZ_ROWS];
            // an Inf or NaN input (exponent bound past the largest finite
            // double's): the vector's far field is not defined
            if (Es[sg * 16 + r] > 1024) bad[v] = 1;
          }
        }
    }
  };
  oz_tile_loop<NBUF>((long long)blockIdx.x * MXW + wid, (long long)gridDim.x * MXW, ntile, issue,
                     work);
}

size_t mz_leaf_up_smem(int KC, int nbuf) {
  return (size_t)(2 * oz_words(OZ_NT, KC) + 2 * OZ_META + 32 * MXW) * 4 +
         (size_t)MXW * nbuf * 16 * (16 * KC + 1) * sizeof(double);
}

// The levels a transfer kernel covers.  One launch per level (TOP = false):
// one level, columns [0, count 2 np) of every tree, tiles over the grid.  The
// top of the trees (TOP = true): levels lv[0], lv[1], ... in the order given
// (up: coarser each step, down: finer), each CTA owning G whole trees, which
// it carries through all those levels with a CTA barrier between levels (a
// level's inputs are the CTA's own outputs of the level before, written to
// global memory and read back by the same SM after the barrier).  The levels
// at the top hold few slots per tree, so one launch replaces several whose
// CTAs would each wait out a single tile's latency.
constexpr int TREE_TOP_MAX = 8;
constexpr int FAR_SPLIT_MAX = 4;  // finest levels whose far field may run on a third stream
struct TreeLevel {
  long long pb, cb, np;  // parent / child slot base of the level, parents per tree
};
struct TreeLevels {
  int n, G;  // levels, trees per CTA (TOP)
  TreeLevel lv[TREE_TOP_MAX];
};

// The per-warp tile loop of a kernel: one level over the grid, or (TOP) the
// CTA's trees through every level.  issue / work take the level and the
// column range [c0, c1) the tile index counts from.
template <bool TOP, int NBUF, class Issue, class Work>
__device__ __forceinline__ void tree_levels_loop(const TreeLevels &T, long long count,
                                                 Issue issue, Work work) {
  const int wid = threadIdx.x >> 5;
  if constexpr (!TOP) {
    const TreeLevel Lv = T.lv[0];
    const long long c1 = count * 2 * Lv.np;
    oz_tile_loop<NBUF>(
        (long long)blockIdx.x * MXW + wid, (long long)gridDim.x * MXW, (c1 + 15) / 16,
        [&](long long t, int b) { issue(Lv, 0LL, c1, t, b); },
        [&](long long t, int b) { work(Lv, 0LL, c1, t, b); });
  } else {
    const long long trees = count * 2, v0 = (long long)blockIdx.x * T.G;
    const long long v1 = v0 + T.G < trees ? v0 + T.G : trees;
    for (int k = 0; k < T.n; k++) {
      const TreeLevel Lv = T.lv[k];
      const long long c0 = v0 * Lv.np, c1 = v1 * Lv.np;
      oz_tile_loop<NBUF>(
          (long long)wid, (long long)MXW, (c1 - c0 + 15) / 16,
          [&](long long t, int b) { issue(Lv, c0, c1, t, b); },
          [&](long long t, int b) { work(Lv, c0, c1, t, b); });
      __syncthreads();  // the level's outputs, in global memory, for the next
    }
  }
}

// Transfer trees.  Columns col = (vector * 2 + parity) * np + j.
// Up: parent slot j of level l from child slots 2j+2, 2j+3 of level l+1
// (36 contiguous coefficients, two stored columns), P = [B | B'] (18 x 36).
// The transfer matrices' fragments hold only their first QMAX digit slices
// (the slice-major layout makes that a prefix of each matrix's words).
__host__ __device__ constexpr int oz_tree_words(int QMAX, int KC) { return QMAX * OZ_NT * KC * 32; }
template <int QMAX, int NBUF, bool TOP = false>
__global__ void __launch_bounds__(32 * MXW, oz_min_ctas(NBUF))
    k_mz_tree_up(long long *w, int *wE, const unsigned *__restrict__ Pf,
                 const int *__restrict__ Pm, Geo g, TreeLevels T) {
  extern __shared__ __align__(16) unsigned char mz_smem[];
  constexpr int NW = oz_tree_words(QMAX, 5);
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
  unsigned *sP = reinterpret_cast<unsigned *>(mz_smem);
  int *sM = reinterpret_cast<int *>(sP + NW);
  // per warp: Es[16], then [buf][child][16] exponents
  int *sI = sM + OZ_META + wid * (16 + NBUF * 2 * 16);
  int *Es = sI, *sEx = sI + 16;
  long long *sB0 = reinterpret_cast<long long *>(sM + OZ_META + MXW * (16 + NBUF * 2 * 16));
  long long *sB = sB0 + wid * NBUF * 16;
  long long *Xw = sB0 + MXW * NBUF * 16 + wid * NBUF * 16 * OZ_TLD;
  oz_load_frag(sP, Pf, NW, sM, Pm, OZ_META);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  auto issue = [&](const TreeLevel &Lv, long long c0, long long c1, long long tile, int buf) {
    const long long np = Lv.np;
    long long *B = sB + buf * 16;
    int *Ex = sEx + buf * 32;
    if (lane < 16) {
      const long long col = c0 + tile * 16 + lane;
      long long b = -1;
      if (col < c1) {
        const long long vs = col / np, j = col - vs * np;
        b = vs * g.slots + Lv.cb + 2 * j + 2;  // first child slot
      }
      B[lane] = b;
      cp_async4(Ex + lane, b >= 0 ? wE + b : wE, b >= 0 ? 4 : 0);
      cp_async4(Ex + 16 + lane, b >= 0 ? wE + b + 1 : wE, b >= 0 ? 4 : 0);
    }
    __syncwarp();
    long long *X = Xw + buf * 16 * OZ_TLD;
    for (int e = lane; e < 16 * M; e += 32) {  // 16 columns x 18 pairs
      const int r = e / M, k2 = e - r * M;
      const long long b = B[r];
      l2c_oz::cp_async16(X + r * OZ_TLD + 2 * k2, b >= 0 ? w + b * M + 2 * k2 : w, b >= 0 ? 16 : 0);
    }
  };
  auto work = [&](const TreeLevel &Lv, long long cb0, long long c1, long long tile, int buf) {
    const long long np = Lv.np;
    long long *X = Xw + buf * 16 * OZ_TLD;
    const int *Ex = sEx + buf * 32;
    l2c_oz::stage_cols<2 * M, M, 40>(X, OZ_TLD, Ex, Ex + 16, Es);
    long long T[OZ_NT][4];
    oz_tile_T<OZ_NT, 5, QMAX>(sP, X, OZ_TLD, 1, T);
    const long long c0 = cb0 + tile * 16;
    auto dst = [&](int r) -> long long {  // parent slot index, -1: none
      const long long col = c0 + r;
      if (col >= c1) return -1;
      const long long vs = col / np, j = col - vs * np;
      return vs * g.slots + Lv.pb + j;
    };
    const long long d0 = dst(gq), d1 = dst(gq + 8);
    oz_put18(
        T, sM,
        [&](int r, int n, long long a, long long b) {
          const long long d = r < 8 ? d0 : d1;
          if (d >= 0) *reinterpret_cast<longlong2 *>(w + d * M + n) = make_longlong2(a, b);
        },
        [&](int r, int n, long long a) {
          const long long d = r < 8 ? d0 : d1;
          if (d >= 0) w[d * M + n] = a;
        });
    if (t4 == 0) {
      if (d0 >= 0) wE[d0] = Es[gq] + sM[OZ_ROWS];
      if (d1 >= 0) wE[d1] = Es[gq + 8] + sM[OZ_ROWS];
    }
  };
  tree_levels_loop<TOP, NBUF>(T, g.count, issue, work);
}

constexpr size_t oz_tree_up_smem(int QMAX, int NBUF) {
  return (size_t)(oz_tree_words(QMAX, 5) + OZ_META + MXW * (16 + NBUF * 2 * 16)) * 4 +
         (size_t)MXW * NBUF * 16 * 8 + (size_t)MXW * NBUF * 16 * OZ_TLD * sizeof(long long);
}

// Down: child slots 2t, 2t+1 of level l+1 += [B^T; B^T'] c(parent slot t of
// level l).  The child's own far field (prefetched with the parent) and the
// product are added as integers on the coarser of their two scales, one bit
// above the larger exponent.
template <int QMAX, int NBUF, bool TOP = false>
__global__ void __launch_bounds__(32 * MXW, oz_min_ctas(NBUF))
    k_mz_tree_down(long long *c, int *cE, const unsigned *__restrict__ Pf,
                   const int *__restrict__ Pm, Geo g, TreeLevels T) {
  extern __shared__ __align__(16) unsigned char mz_smem[];
  constexpr int NW = oz_tree_words(QMAX, 3);  // per matrix: B^T, then B^T'
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
  unsigned *sP = reinterpret_cast<unsigned *>(mz_smem);
  int *sM = reinterpret_cast<int *>(sP + 2 * NW);
  // per warp: Es[16], then per buffer: parent exponent [16], child exponents [2][16]
  int *sI = sM + 2 * OZ_META + wid * (16 + NBUF * 3 * 16);
  int *Es = sI, *sEx = sI + 16;
  long long *sB0 = reinterpret_cast<long long *>(sM + 2 * OZ_META + MXW * (16 + NBUF * 3 * 16));
  long long *sB = sB0 + wid * NBUF * 2 * 16;  // [buf][parent | child][16] slot indices
  long long *X0 = sB0 + MXW * NBUF * 2 * 16;
  long long *Xw = X0 + wid * NBUF * 16 * OZ_CLD;
  long long *Cw = X0 + MXW * NBUF * 16 * OZ_CLD + wid * NBUF * 16 * 2 * M;
  oz_load_frag(sP, Pf, 2 * NW, sM, Pm, 2 * OZ_META);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  auto issue = [&](const TreeLevel &Lv, long long c0, long long c1, long long tile, int buf) {
    const long long np = Lv.np;
    long long *B = sB + buf * 32;
    int *Ex = sEx + buf * 48;
    if (lane < 16) {
      const long long col = c0 + tile * 16 + lane;
      long long b = -1, cb = -1;
      if (col < c1) {
        const long long vs = col / np, t = col - vs * np;
        b = vs * g.slots + Lv.pb + t;
        cb = vs * g.slots + Lv.cb + 2 * t;
      }
      B[lane] = b;
      B[16 + lane] = cb;
      cp_async4(Ex + lane, b >= 0 ? cE + b : cE, b >= 0 ? 4 : 0);
      cp_async4(Ex + 16 + lane, cb >= 0 ? cE + cb : cE, cb >= 0 ? 4 : 0);
      cp_async4(Ex + 32 + lane, cb >= 0 ? cE + cb + 1 : cE, cb >= 0 ? 4 : 0);
    }
    __syncwarp();
    long long *X = Xw + buf * 16 * OZ_CLD, *C = Cw + buf * 16 * 2 * M;
    for (int e = lane; e < 16 * (M / 2); e += 32) {  // 16 parent columns x 9 pairs
      const int r = e / (M / 2), k2 = e - r * (M / 2);
      const long long b = B[r];
      l2c_oz::cp_async16(X + r * OZ_CLD + 2 * k2, b >= 0 ? c + b * M + 2 * k2 : c, b >= 0 ? 16 : 0);
    }
    for (int e = lane; e < 16 * M; e += 32) {  // 16 child pairs x 18 pairs
      const int r = e / M, k2 = e - r * M;
      const long long b = B[16 + r];
      l2c_oz::cp_async16(C + r * 2 * M + 2 * k2, b >= 0 ? c + b * M + 2 * k2 : c, b >= 0 ? 16 : 0);
    }
  };
  auto work = [&](const TreeLevel &, long long, long long, long long, int buf) {
    long long *X = Xw + buf * 16 * OZ_CLD;
    const long long *C = Cw + buf * 16 * 2 * M;
    const long long *B = sB + buf * 32;
    const int *Ex = sEx + buf * 48;
    l2c_oz::stage_cols<M, M, 24>(X, OZ_CLD, Ex, Ex, Es);
    const long long cb0 = B[16 + gq], cb1 = B[16 + gq + 8];
    // the parent's digits once, for both children's products
    l2c_oz::Digits<3> D;
    l2c_oz::load_digits<3>(X, OZ_CLD, 1, D);
#pragma unroll 1
    for (int ch = 0; ch < 2; ch++) {
      const int *meta = sM + ch * OZ_META;
      // per tile row r: product exponent, child exponent, sum exponent
      int ep[2], ek[2], es[2];
#pragma unroll
      for (int hr = 0; hr < 2; hr++) {
        const int r = gq + 8 * hr;
        ep[hr] = Es[r] + meta[OZ_ROWS];
        ek[hr] = Ex[16 + 16 * ch + r];
        es[hr] = max(ep[hr], ek[hr]) + 1;
      }
      auto sum = [&](int r, int n, long long v) -> long long {
        const int hr = r >> 3;
        return l2c_oz::shift_s64(C[r * 2 * M + ch * M + n], ek[hr] - es[hr]) +
               l2c_oz::shift_s64(v, ep[hr] - es[hr]);
      };
      auto put2 = [&](int r, int n, long long a, long long b) {
        const long long d = r < 8 ? cb0 : cb1;
        if (d >= 0)
          *reinterpret_cast<longlong2 *>(c + (d + ch) * M + n) =
              make_longlong2(sum(r, n, a), sum(r, n + 1, b));
      };
      auto put1 = [&](int r, int n, long long a) {
        const long long d = r < 8 ? cb0 : cb1;
        if (d >= 0) c[(d + ch) * M + n] = sum(r, n, a);
      };
#pragma unroll
      for (int nt = 0; nt < OZ_NT; nt++) {
        float acc[l2c_oz::NDIAG][4];
        l2c_oz::mma_nt<OZ_NT, 3, QMAX>(sP + ch * NW, D, nt, acc);
        long long T4[4];
#pragma unroll
        for (int e = 0; e < 4; e++) T4[e] = l2c_oz::combine1(acc, e);
        oz_put_nt(nt, T4, meta, put2, put1);
      }
      if (t4 == 0) {
        if (cb0 >= 0) cE[cb0 + ch] = es[0];
        if (cb1 >= 0) cE[cb1 + ch] = es[1];
      }
    }
  };
  tree_levels_loop<TOP, NBUF>(T, g.count, issue, work);
}

constexpr size_t oz_tree_down_smem(int QMAX, int NBUF) {
  return (size_t)(2 * oz_tree_words(QMAX, 3) + 2 * OZ_META + MXW * (16 + NBUF * 3 * 16)) * 4 +
         (size_t)MXW * NBUF * 2 * 16 * 8 +
         (size_t)MXW * NBUF * 16 * (OZ_CLD + 2 * M) * sizeof(long long);
}

// Far field (step 3): CTA = (block gb, chunk of columns vs = vector * 2 +
// parity).  c0 = [A0 A1] [w0; w1] and c1 = A2 w1 as one product of the 40-row
// matrix of k_oz_pack_far with the column [w0; w1] (K = 36), on the scale of
// the whole column: the same integers as two products over the same staged
// words, with the digits extracted once.  A CTA takes cols columns (a
// multiple of 16 MXW: one or two 16-column tiles per warp, in turn).
constexpr int OZ_FAR_COLS = 16 * MXW * 2;  // columns per CTA (at most)
// Far-field blocks gb0 + blockIdx.x (a launch may cover one level's blocks).
template <int NBUF>
__global__ void __launch_bounds__(32 * MXW, oz_min_ctas(NBUF))
    k_mz_far(const long long *__restrict__ w, const int *__restrict__ wE, long long *__restrict__ c,
             int *__restrict__ cE, const unsigned *__restrict__ Pf, const int *__restrict__ Pm,
             Geo g, long long gb0, int cols) {
  extern __shared__ __align__(16) unsigned char mz_smem[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
  unsigned *sP = reinterpret_cast<unsigned *>(mz_smem);
  int *sM = reinterpret_cast<int *>(sP + OZ_FAR_WORDS);
  int *sI = sM + 2 * OZ_META + wid * (16 + NBUF * 2 * 16);  // Es[16], [buf][slot][16]
  int *Es = sI, *sEx = sI + 16;
  long long *Xw = reinterpret_cast<long long *>(sM + 2 * OZ_META + MXW * (16 + NBUF * 2 * 16)) +
                  wid * NBUF * 16 * OZ_TLD;
  const long long gb = gb0 + blockIdx.x;
  oz_load_frag(sP, Pf + gb * OZ_FAR_WORDS, OZ_FAR_WORDS, sM, Pm + gb * 2 * OZ_META, 2 * OZ_META);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  const long long ncol = 2 * g.count, c0 = (long long)blockIdx.y * cols;
  const long long ntile = (min(ncol - c0, (long long)cols) + 15) / 16;
  auto issue = [&](long long tile, int buf) {
    long long *X = Xw + buf * 16 * OZ_TLD;
    int *Ex = sEx + buf * 32;
    if (lane < 16) {
      const long long col = c0 + tile * 16 + lane;
      const bool ok = col < ncol;
      cp_async4(Ex + lane, ok ? wE + col * g.slots + 2 * gb : wE, ok ? 4 : 0);
      cp_async4(Ex + 16 + lane, ok ? wE + col * g.slots + 2 * gb + 1 : wE, ok ? 4 : 0);
    }
    for (int e = lane; e < 16 * M; e += 32) {  // 16 columns x 18 pairs
      const int r = e / M, k2 = e - r * M;
      const long long col = c0 + tile * 16 + r;
      const bool ok = col < ncol;
      l2c_oz::cp_async16(X + r * OZ_TLD + 2 * k2, ok ? w + (col * g.slots + 2 * gb) * M + 2 * k2 : w,
                         ok ? 16 : 0);
    }
  };
  auto work = [&](long long tile, int buf) {
    long long *X = Xw + buf * 16 * OZ_TLD;
    const int *Ex = sEx + buf * 32;
    l2c_oz::stage_cols<2 * M, M, OZ_TLD>(X, OZ_TLD, Ex, Ex + 16, Es);
    const long long cA = c0 + tile * 16 + gq, cB = cA + 8;
    // the tile's digits once, then the 40-row product one n-tile at a time;
    // n-tiles 3 and 4 (rows 24 .. 39, the second slot's) have zero weights on
    // the first slot's moments (chunk pair 0)
    l2c_oz::Digits<OZ_FAR_KC> D;
    l2c_oz::load_digits<OZ_FAR_KC>(X, OZ_TLD, 1, D);
#pragma unroll
    for (int nt = 0; nt < OZ_FAR_NT; nt++) {
      float acc[l2c_oz::NDIAG][4];
      if (nt < 3)
        l2c_oz::mma_nt<OZ_FAR_NT, OZ_FAR_KC>(sP, D, nt, acc);
      else
        l2c_oz::mma_nt<OZ_FAR_NT, OZ_FAR_KC, l2c_oz::SLICES, 1>(sP, D, nt, acc);
      // the lane's outputs: rows n, n + 1 of data columns cA (e = 0, 1) and
      // cB (e = 2, 3); rows 0 .. 17 go to slot 2 gb, 18 .. 35 to 2 gb + 1
      const int n = 8 * nt + 2 * t4;
      if (n < 2 * M) {
        const int part = n >= M ? 1 : 0, r = n - part * M;
        const int *meta = sM + part * OZ_META;
#pragma unroll
        for (int hr = 0; hr < 2; hr++) {
          const long long col = hr ? cB : cA;
          const long long V0 = l2c_oz::shift_s64(l2c_oz::combine1(acc, 2 * hr), meta[r]);
          const long long V1 = l2c_oz::shift_s64(l2c_oz::combine1(acc, 2 * hr + 1), meta[r + 1]);
          if (col < ncol)
            *reinterpret_cast<longlong2 *>(c + (col * g.slots + 2 * gb + part) * M + r) =
                make_longlong2(V0, V1);
        }
      }
    }
    if (t4 == 0)
#pragma unroll
      for (int part = 0; part < 2; part++) {
        const int eo = sM[part * OZ_META + OZ_ROWS];
        if (cA < ncol) cE[cA * g.slots + 2 * gb + part] = Es[gq] + eo;
        if (cB < ncol) cE[cB * g.slots + 2 * gb + part] = Es[gq + 8] + eo;
      }
  };
  oz_tile_loop<NBUF>(wid, MXW, ntile, issue, work);
}

constexpr size_t oz_far_smem(int NBUF) {
  return (size_t)(OZ_FAR_WORDS + 2 * OZ_META + MXW * (16 + NBUF * 2 * 16)) * 4 +
         (size_t)MXW * NBUF * 16 * OZ_TLD * sizeof(long long);
}

// Far field on the fifth-generation tensor cores (TuneCfg::fartc): the product
// of k_mz_far -- the 40-row block matrix of k_oz_pack_far times the columns
// [w0; w1] -- with the diagonal sums accumulated in tensor memory instead of
// registers.  CTA = (block gb, 128 columns vs = vector * 2 + parity): column m
// of the CTA is row m of an M = 128, N = 48 MMA (output rows 0 .. 47).  Its two
// slots' moments (18 + 18) sit at K positions 0 .. 17 and 24 .. 41 of three
// 16-wide k-steps; the other K positions are zero, as are the packed matrix's
// there (k_oz_pack_far_tc).  One MMA per digit pair and k-step: each reads its
// 128-row operand tile from shared memory once, so few wide products cost
// less than many narrow ones.  The six diagonals are formed in three passes of
// two (d = 2 pass, 2 pass + 1: 3, 7 and 11 digit pairs) into two tensor-memory
// buffers of 128 columns (diagonal 2 pass + e at 128 (pass % 2) + 64 e), so a
// pass is read out while the next one multiplies; each lane adds its outputs'
// share of the combination (l2c_oz::combine6, split by diagonal pairs) in
// 64-bit registers.  Every diagonal sum is the same integer as k_mz_far's (the
// accumulation is exact), so are the outputs.  The digits of the columns are
// written to shared memory in the K-major no-swizzle layout of l2c_tc.cuh, the
// block matrix's arrive by one bulk copy.
constexpr int FTC_COLS = 128, FTC_THREADS = 256;
constexpr uint32_t FTC_A_BYTES = l2c_oz::SLICES * 3 * 4096;  // digits of 128 columns
constexpr uint32_t FTC_B_BYTES = l2c_oz::SLICES * 3 * 1536;  // digits of the 48-row matrix
constexpr int FTC_B_WORDS = (int)(FTC_B_BYTES / 4);
constexpr uint32_t FTC_TMEM_COLS = 256;  // two buffers of two diagonals
constexpr size_t ftc_smem() {
  return FTC_A_BYTES + FTC_B_BYTES + 2 * OZ_META * 4 + 4 * 8 + 16;
}
// Tensor memory holds 512 columns per SM: with more than a third of the SM's
// 228 KB of shared memory per CTA, at most two of these CTAs are resident on
// an SM, and their allocations always fit (an allocation never waits).
static_assert(3 * (ftc_smem() + 1024) > 228 * 1024, "a third CTA could wait for tensor memory");
static_assert(2 * (ftc_smem() + 1024) <= 228 * 1024, "two CTAs per SM");

// Far-field block fragments in k_mz_far_tc's operand layout, from the words of
// k_oz_pack_far (the same digits): per block FTC_B_WORDS words; the FP16 pair
// at K positions (kp, kp + 1) of row n, digit slice q, lies in k-step
// ks = kp / 16 at byte ((q - 1) 3 + ks) 1536 + l2c_tc::tile_offset(n, kp % 16).
// K position kp holds moment kp (kp < 18) or kp - 6 (24 <= kp < 42), zero
// elsewhere; rows 40 .. 47 are zero.  One thread per word.
__global__ void k_oz_pack_far_tc(const unsigned *__restrict__ F, long long nblocks,
                                 unsigned *__restrict__ Ft) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= nblocks * FTC_B_WORDS) return;
  const long long gb = idx / FTC_B_WORDS;
  const int off = 4 * (int)(idx - gb * FTC_B_WORDS);
  const int reg = off / 1536, in = off - reg * 1536;
  const int q = reg / 3 + 1, ks = reg % 3;
  const int n = (in / 256) * 8 + (in % 128) / 16;
  const int kp = ks * 16 + ((in % 256) / 128) * 8 + (in % 16) / 2;
  const int k = kp < M ? kp : (kp >= 24 && kp < 24 + M ? kp - 6 : -1);
  unsigned v = 0u;
  if (n < 8 * OZ_FAR_NT && k >= 0)
    v = F[gb * OZ_FAR_WORDS + l2c_oz::frag_index(q, n / 8, k / 8, 4 * (n % 8) + (k % 8) / 2,
                                                 OZ_FAR_NT, OZ_FAR_KC)];
  Ft[idx] = v;
}

// Read-out of pass P for the lane's column: the FP32 sums of diagonals 2P and
// 2P + 1 of outputs N0 .. N0 + 2 NW - 1 at tensor-memory columns ta + [0, 2 NW)
// and ta + 64 + [0, 2 NW); those in [NB, NB + 18) add their share of
// l2c_oz::combine6 to T[n - NB] (modulo 2^64, as combine6 forms it).
template <int P, int NW, int N0, int NB>
__device__ __forceinline__ void ftc_pass_chunk(uint32_t ta, long long (&T)[M]) {
  uint32_t r[2][2 * NW];
#pragma unroll
  for (int e = 0; e < 2; e++) {
    if constexpr (NW == 4) {
      l2c_tc::tmem_ld8(ta + 64 * e, *reinterpret_cast<uint32_t(*)[8]>(r[e]));
    } else if constexpr (NW == 2) {
      l2c_tc::tmem_ld4(ta + 64 * e, *reinterpret_cast<uint32_t(*)[4]>(r[e]));
    } else {
      l2c_tc::tmem_ld2(ta + 64 * e, *reinterpret_cast<uint32_t(*)[2]>(r[e]));
    }
  }
  l2c_tc::tmem_ld_wait();
#pragma unroll
  for (int j = 0; j < 2 * NW; j++) {
    const int n = N0 + j;
    if (n >= NB && n < NB + M) {
      const int a = __float2int_rn(__uint_as_float(r[0][j]));
      const int b = __float2int_rn(__uint_as_float(r[1][j]));
      long long &t = T[(n - NB) % M];
      if constexpr (P == 0) {
        t = (long long)((unsigned long long)((long long)b * (1 << 27)) +
                        ((unsigned long long)((unsigned)a << 4) << 32));
      } else if constexpr (P == 1) {
        t += (long long)a * (1 << 18) + (long long)b * (1 << 9);
      } else {
        t += (long long)(a + (b >> 9));
      }
    }
  }
}

// Pass P's read-out for the lane (half 0: outputs 0 .. 17, half 1: 18 .. 35)
// from the buffer at tensor-memory address ta.
template <int P>
__device__ __forceinline__ void ftc_pass(uint32_t ta, int half, long long (&T)[M]) {
  if (half == 0) {
    ftc_pass_chunk<P, 4, 0, 0>(ta + 0, T);
    ftc_pass_chunk<P, 4, 8, 0>(ta + 8, T);
    ftc_pass_chunk<P, 1, 16, 0>(ta + 16, T);
  } else {
    ftc_pass_chunk<P, 4, 16, M>(ta + 16, T);
    ftc_pass_chunk<P, 4, 24, M>(ta + 24, T);
    ftc_pass_chunk<P, 2, 32, M>(ta + 32, T);
  }
}

// The MMAs of pass P (diagonals 2P and 2P + 1, all 48 output rows) into the
// buffer at tensor-memory column tbuf: diagonal 2P + e at tbuf + 64 e.
template <int P>
__device__ __forceinline__ void ftc_issue(uint32_t tbuf, const unsigned char *sA,
                                          const unsigned char *sB) {
  const uint32_t id = l2c_tc::idesc_f16_f32(128, 48);
#pragma unroll 1
  for (int ks = 0; ks < 3; ks++)
#pragma unroll
    for (int q = 1; q <= l2c_oz::SLICES; q++) {
      const uint64_t bd = l2c_tc::smem_desc(l2c_tc::smem_u32(sB + ((q - 1) * 3 + ks) * 1536),
                                            l2c_tc::CORE_LBO, l2c_tc::CORE_SBO);
#pragma unroll
      for (int p = 1; p + q <= l2c_oz::DMAX; p++) {
        const int e = p + q - 2 - 2 * P;
        if (e == 0 || e == 1)
          l2c_tc::mma_f16(tbuf + 64 * e,
                          l2c_tc::smem_desc(l2c_tc::smem_u32(sA + ((p - 1) * 3 + ks) * 4096),
                                            l2c_tc::CORE_LBO, l2c_tc::CORE_SBO),
                          bd, id, (ks > 0 || q > 1) ? 1u : 0u);
      }
    }
}

// Far-field blocks gb0 + blockIdx.x, columns 128 blockIdx.y ...  The tensor
// memory is allocated once the CTA's operands are staged, after the grid
// dependency wait (a CTA never holds it while waiting on another grid), and
// two CTAs' allocations fit an SM's tensor memory.  Every mbarrier wait is bounded (about a second); when one runs out the CTA
// waits (bounded) for its copy and products in flight, marks its vectors in
// bad (their outputs become NaN) and frees its tensor memory.
__global__ void __launch_bounds__(FTC_THREADS, 2)
    k_mz_far_tc(const long long *__restrict__ w, const int *__restrict__ wE,
                long long *__restrict__ c, int *__restrict__ cE, const unsigned *__restrict__ Pt,
                const int *__restrict__ Pm, Geo g, long long gb0, int *__restrict__ bad) {
  extern __shared__ __align__(16) unsigned char mz_smem[];
  unsigned char *sA = mz_smem, *sB = sA + FTC_A_BYTES;
  int *sM = reinterpret_cast<int *>(sB + FTC_B_BYTES);
  // bars: [0] the matrix copy, [1] [2] the products of the two buffers,
  // [3] everything issued (error path)
  uint64_t *bars = reinterpret_cast<uint64_t *>(sM + 2 * OZ_META);
  uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 4);
  volatile int *s_err = reinterpret_cast<volatile int *>(slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long gb = gb0 + blockIdx.x;
  const long long ncol = 2 * g.count, c0 = (long long)blockIdx.y * FTC_COLS;
  if (tid == 0) {
    for (int i = 0; i < 4; i++) l2c_tc::bar_init(&bars[i], 1);
    *s_err = 0;
    l2c_tc::bar_init_fence();
  }
  __syncthreads();
  if (tid == 0) l2c_tc::bulk_load(sB, Pt + gb * FTC_B_WORDS, FTC_B_BYTES, &bars[0]);
  for (int i = tid; i < 2 * OZ_META; i += FTC_THREADS) sM[i] = Pm[gb * 2 * OZ_META + i];
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  {
    // Staging as l2c_oz::stage_cols does it: two threads per column (lanes
    // r and r + 16), thread h holding slot 2 gb + h's 18 moments in registers;
    // then the six digit slices into the operand tile.
    const int m = warp * 16 + (lane & 15), h = lane >> 4;
    const long long col = c0 + m;
    const bool ok = col < ncol;
    long long v[M];
    int e = 0;
    if (ok) {
      const longlong2 *src =
          reinterpret_cast<const longlong2 *>(w + (col * g.slots + 2 * gb + h) * M);
#pragma unroll
      for (int i = 0; i < M / 2; i++) {
        const longlong2 t = src[i];
        v[2 * i] = t.x;
        v[2 * i + 1] = t.y;
      }
      e = wE[col * g.slots + 2 * gb + h];
    } else {
#pragma unroll
      for (int i = 0; i < M; i++) v[i] = 0;
    }
    const int ec = max(e, __shfl_xor_sync(0xffffffffu, e, 16));
    unsigned long long mx = 0;
#pragma unroll
    for (int i = 0; i < M; i++) {
      v[i] = l2c_oz::shift_s64(v[i], e - ec);
      const unsigned long long a =
          v[i] < 0 ? 0ull - (unsigned long long)v[i] : (unsigned long long)v[i];
      mx = a > mx ? a : mx;
    }
    const unsigned long long mo = __shfl_xor_sync(0xffffffffu, mx, 16);
    mx = mo > mx ? mo : mx;
    const int B = 64 - __clzll((long long)mx);
    const int sh = l2c_oz::FRAC - B;
    l2c_oz::Ysplit ys[M];
#pragma unroll
    for (int i = 0; i < M; i++)
      ys[i] = l2c_oz::ysplit((sh >= 0 ? v[i] << sh : v[i] >> -sh) + l2c_oz::RBAL);
    if (ok) cE[col * g.slots + 2 * gb + h] = ec - l2c_oz::VBITS + B + sM[h * OZ_META + OZ_ROWS];
    // K group 3 h + j (8 positions) of row m: k-step (3 h + j) / 2, half (3 h + j) % 2
    unsigned char *row = sA + (m >> 3) * l2c_tc::CORE_SBO + (m & 7) * 16;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int grp = 3 * h + j;
      unsigned char *dst = row + (grp >> 1) * 4096 + (grp & 1) * l2c_tc::CORE_LBO;
#define L2C_FTC_SLICE(P)                                                         \
  {                                                                              \
    uint4 u;                                                                     \
    if (j < 2) {                                                                 \
      u.x = l2c_oz::dig2<P>(ys[8 * j], ys[8 * j + 1]);                           \
      u.y = l2c_oz::dig2<P>(ys[8 * j + 2], ys[8 * j + 3]);                       \
      u.z = l2c_oz::dig2<P>(ys[8 * j + 4], ys[8 * j + 5]);                       \
      u.w = l2c_oz::dig2<P>(ys[8 * j + 6], ys[8 * j + 7]);                       \
    } else {                                                                     \
      u.x = l2c_oz::dig2<P>(ys[M - 2], ys[M - 1]);                               \
      u.y = u.z = u.w = 0u;                                                      \
    }                                                                            \
    *reinterpret_cast<uint4 *>(dst + (P - 1) * 3 * 4096) = u;                    \
  }
      L2C_FTC_SLICE(1) L2C_FTC_SLICE(2) L2C_FTC_SLICE(3)
      L2C_FTC_SLICE(4) L2C_FTC_SLICE(5) L2C_FTC_SLICE(6)
#undef L2C_FTC_SLICE
    }
  }
  l2c_tc::fence_async_smem();
  __syncthreads();
  if (warp == 0) l2c_tc::tmem_alloc(slot, FTC_TMEM_COLS);
  l2c_tc::fence_before_sync();
  __syncthreads();
  l2c_tc::fence_after_sync();
  const uint32_t tb = *slot;
  // bars[1] / bars[2]: the products of buffer 0 (passes 0 and 2) / buffer 1 (pass 1)
  bool issued = false;
  if (tid == 0) {
    if (!l2c_tc::bar_wait(&bars[0], 0)) {
      *s_err = 1;
    } else {
      ftc_issue<0>(tb, sA, sB);
      l2c_tc::mma_commit(&bars[1]);
      ftc_issue<1>(tb + 128, sA, sB);
      l2c_tc::mma_commit(&bars[2]);
      issued = true;
    }
  }
  __syncthreads();
  // Reading out: warp w reads tensor-memory lanes 32 (w % 4) .. + 31 (columns
  // m of the CTA); warps 0 .. 3 the first slot's rows 0 .. 17, warps 4 .. 7
  // the second slot's, 18 .. 35.
  const int q4 = warp & 3, half = warp >> 2;
  const long long col = c0 + 32 * q4 + lane;
  const uint32_t ta = tb + ((uint32_t)(32 * q4) << 16);
  long long T[M];
  bool ok = *s_err == 0;
  ok = __all_sync(0xffffffffu, ok && l2c_tc::bar_wait(&bars[1], 0));
  if (ok) {
    l2c_tc::fence_after_sync();
    ftc_pass<0>(ta, half, T);
  } else {
    *s_err = 1;
  }
  l2c_tc::fence_before_sync();
  __syncthreads();
  ok = ok && *s_err == 0;
  if (tid == 0 && ok) {
    l2c_tc::fence_after_sync();
    ftc_issue<2>(tb, sA, sB);
    l2c_tc::mma_commit(&bars[1]);
  }
  ok = __all_sync(0xffffffffu, ok && l2c_tc::bar_wait(&bars[2], 0));
  if (ok) {
    l2c_tc::fence_after_sync();
    ftc_pass<1>(ta + 128, half, T);
  }
  ok = __all_sync(0xffffffffu, ok && l2c_tc::bar_wait(&bars[1], 1));
  if (ok) {
    l2c_tc::fence_after_sync();
    ftc_pass<2>(ta, half, T);
    if (col < ncol) {
      const int *meta = sM + half * OZ_META;
      long long *out = c + (col * g.slots + 2 * gb + half) * M;
#pragma unroll
      for (int i = 0; i < M; i += 2)
        *reinterpret_cast<longlong2 *>(out + i) = make_longlong2(
            l2c_oz::shift_s64(T[i], meta[i]), l2c_oz::shift_s64(T[i + 1], meta[i + 1]));
    }
  } else {
    *s_err = 1;
  }
  l2c_tc::fence_before_sync();
  __syncthreads();
  if (*s_err != 0) {
    if (tid == 0) {
      l2c_tc::bar_wait(&bars[0], 0);
      if (issued) {
        l2c_tc::mma_commit(&bars[3]);
        l2c_tc::bar_wait(&bars[3], 0);
      }
    }
    if (tid < FTC_COLS && c0 + tid < ncol) bad[(c0 + tid) >> 1] = 1;
  }
  if (warp == 0) {
    __syncwarp();
    l2c_tc::fence_after_sync();
    l2c_tc::tmem_dealloc(tb, FTC_TMEM_COLS);
  }
}

// Leaf down (step 5) + final scaling: tile = 16 consecutive leaf targets of one
// vector, both parities; P_sg = T_sg (s x 18) in passes of 16 output rows
// (two n-tiles, KC = 3).  For tile row r, pass ps and parity sg a lane quad
// holds the far field of outputs (tau0 + r) h + 32 ps + 2 [0, 16) + sg (lane
// t: 4t + {0, 2} and 16 + 4t + {0, 2}): every other output.  The warp stages
// both parities' far field of its 16 rows in shared memory (rows of h + 1
// doubles), then reads y and writes the scaled sums a whole row at a time, so
// loads and stores are contiguous -- full sectors also when the output is
// page-locked host memory written over the host link.  The outputs past the
// last leaf target (band only) are scaled by the same CTAs.
constexpr int OZ_LD_WORDS = oz_words(2, 3);
template <int NBUF>
__global__ void __launch_bounds__(32 * MXW, NBUF == 1 ? 4 : 1)
    k_mz_leaf_down(const long long *__restrict__ c, const int *__restrict__ cE,
                   const double *__restrict__ y, double *out, const unsigned *__restrict__ Pf,
                   const int *__restrict__ Pe, Geo g, int c2l, int npass,
                   const int *__restrict__ bad) {
  extern __shared__ __align__(16) unsigned char mz_smem[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
  const int nw = 2 * npass * OZ_LD_WORDS, ne = 2 * npass * 16;
  unsigned *sP = reinterpret_cast<unsigned *>(mz_smem);
  int *sE = reinterpret_cast<int *>(sP + nw);
  int *Ec = sE + ne + wid * (32 + NBUF * 32);  // Ec[2][16], then [buf][parity][16] exponents
  int *sEx = Ec + 32;
  long long *X0 = reinterpret_cast<long long *>(sE + ne + MXW * (32 + NBUF * 32));
  long long *Xw = X0 + wid * NBUF * 2 * 16 * OZ_CLD;
  const int sld = (int)g.h + 1;  // staged far field: [16][h + 1] doubles per warp
  double *S = reinterpret_cast<double *>(X0 + MXW * NBUF * 2 * 16 * OZ_CLD) + wid * 16 * sld;
  oz_load_frag(sP, Pf, nw, sE, Pe, ne);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  auto scale = [&](double val, long long j) -> double {
    if (!c2l) {
      val = val * l2c_out_scale(j);
    } else {
      val = val * dyadic(2 * (unsigned long long)j + 1, -1);  // j + 1/2
    }
    return val;
  };
  const long long tpv = (g.K + 15) / 16, ntile = g.count * tpv;
  auto issue = [&](long long tile, int buf) {
    const long long v = tile / tpv, tau0 = (tile - v * tpv) * 16;
    const long long nrow = min(16LL, g.K - tau0);
    long long *X = Xw + buf * 2 * 16 * OZ_CLD;
    int *Ex = sEx + buf * 32;
    {
      const int sg = lane >> 4, r = lane & 15;
      const bool ok = r < nrow;
      const long long slot = (v * 2 + sg) * g.slots + g.leaf_base + tau0 + r;
      cp_async4(Ex + lane, ok ? cE + slot : cE, ok ? 4 : 0);
    }
    for (int e = lane; e < 2 * 16 * (M / 2); e += 32) {  // 2 parities x 16 rows x 9 pairs
      const int sr = e / (M / 2), k2 = e - sr * (M / 2), sg = sr >> 4, r = sr & 15;
      const bool ok = r < nrow;
      const long long *src = c + ((v * 2 + sg) * g.slots + g.leaf_base + tau0 + r) * M + 2 * k2;
      l2c_oz::cp_async16(X + sr * OZ_CLD + 2 * k2, ok ? src : c, ok ? 16 : 0);
    }
  };
  auto work = [&](long long tile, int buf) {
    const long long v = tile / tpv, tau0 = (tile - v * tpv) * 16;
    const long long nrow = min(16LL, g.K - tau0);
    const int *Ex = sEx + buf * 32;
#pragma unroll 1
    for (int sg = 0; sg < 2; sg++) {
      long long *X = Xw + (buf * 2 + sg) * 16 * OZ_CLD;
      l2c_oz::stage_cols<M, M, 24>(X, OZ_CLD, Ex + 16 * sg, Ex + 16 * sg, Ec + 16 * sg);
      l2c_oz::Digits<3> D;
      l2c_oz::load_digits<3>(X, OZ_CLD, 1, D);
#pragma unroll 1
      for (int ps = 0; ps < npass; ps++) {
        const int *Ep = sE + (sg * npass + ps) * 16;
#pragma unroll
        for (int nt = 0; nt < 2; nt++) {
          float acc[l2c_oz::NDIAG][4];
          l2c_oz::mma_nt<2, 3>(sP + (sg * npass + ps) * OZ_LD_WORDS, D, nt, acc);
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const int r = gq + 8 * (e >> 1), il = 8 * nt + 2 * t4 + (e & 1), i = 16 * ps + il;
            if (r >= nrow || i >= g.s) continue;
            S[r * sld + 2 * i + sg] =
                l2c_oz::to_double(l2c_oz::combine1(acc, e), Ec[16 * sg + r] - 52 + Ep[il]);
          }
        }
      }
    }
    __syncwarp();
    const double *yv = y + v * g.N;
    double *ov = out + v * g.dist;
    // a vector with an Inf or NaN input: NaN far field (the FP64 form's NaN
    // reaches the outputs the bad input's blocks interact with)
    const bool nan_v = bad[v] != 0;
    const double qnan = __longlong_as_double(0x7ff8000000000000ll);
    for (long long q = lane; q < g.h; q += 32) {
      // the 16 rows' band sums first (one latency), then the sums
      double yy[16];
#pragma unroll
      for (int r = 0; r < 16; r++) {
        const long long j = (tau0 + r) * g.h + q;
        // the last leaf targets run past N when N < Nn - 2h (K h > N)
        yy[r] = (r < nrow && j < g.N) ? yv[j] : 0.0;
      }
#pragma unroll
      for (int r = 0; r < 16; r++) {
        const long long j = (tau0 + r) * g.h + q;
        if (r < nrow && j < g.N)
          ov[j * g.stride] = scale(yy[r] + (nan_v ? qnan : S[r * sld + q]), j);
      }
    }
    __syncwarp();
  };
  oz_tile_loop<NBUF>((long long)blockIdx.x * MXW + wid, (long long)gridDim.x * MXW, ntile, issue,
                     work);
  // outputs past the last leaf target node: band sum only
  const long long jt = g.K * g.h, ntail = jt < g.N ? g.N - jt : 0;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < g.count * ntail;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long v = idx / ntail, j = jt + (idx - v * ntail);
    out[v * g.dist + j * g.stride] = scale(y[v * g.N + j], j);
  }
}

size_t mz_leaf_down_smem(int npass, int nbuf, long long h) {
  return (size_t)(2 * npass * OZ_LD_WORDS + 2 * npass * 16 + MXW * (32 + nbuf * 32)) * 4 +
         (size_t)MXW * nbuf * 2 * 16 * OZ_CLD * 8 + (size_t)MXW * 16 * (h + 1) * 8;
}

// ---------------------------------------------------------------------------
// Mixed form, batches at s = 16: the near-field band of the full blocks on the
// tensor cores.  Block b and parity p: outputs j = b h + 2 i' + p (i' < s) from
// the window x[v][b h + 2 m' + p] (m' < 2s) through W'[m'][i'] =
// near_weight(m' - i', j) (zero where m' < i'; k_band_tile's table), i.e. the
// product of P = W'^T (s x 2s) with a column per vector, exact in integers
// (l2c_ozaki.cuh: K = 32 terms) and rounded once: y = out_in + P x.  A warp
// takes 16 vectors of one block: their windows (2h = 64 doubles each, both
// parities) are staged once, normalised per vector and parity (stage_fix), and
// give both parities' products; the sums are staged back over the consumed
// words and written a row of h outputs at a time.  The last (ragged) block
// keeps the FP64 sums of k_near (k_mz_band_last).  Error: a few units of 2^-53
// |W'|_row |x|_window per output, the order of the FP64 band's own rounding.
// ---------------------------------------------------------------------------
constexpr int MB_S = 16;                         // the leaf size of this form
constexpr int MB_NT = 2, MB_KC = 4;              // s = 16 outputs, 2s = 32 terms
constexpr int MB_WORDS = oz_words(MB_NT, MB_KC);  // one (block, parity) matrix
constexpr int MB_XLD = 4 * MB_S + 1;             // a staged window of 2h = 64, padded

// Plan time: the fragments F[(b 2 + p) MB_WORDS ..] and row exponents
// Fe[(b 2 + p) 16 + i'] of P for the full blocks b < nL - 1.  One thread per
// (block, parity, row).
__global__ void k_oz_pack_band(const double *__restrict__ a, const double *__restrict__ an,
                               const double *__restrict__ dn, Geo g, int c2l,
                               unsigned *__restrict__ F, int *__restrict__ Fe) {
  const long long n = (g.nL - 1) * 2 * MB_S;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const long long bp = idx / MB_S;
  const int ip = (int)(idx - bp * MB_S);
  const long long b = bp >> 1, p = bp & 1, j = b * g.h + 2 * ip + p;
  oz_pack_row([&](int mp) { return mp >= ip ? near_weight(c2l, mp - ip, j, a, an, dn) : 0.0; },
              true, ip, 2 * MB_S, MB_NT, MB_KC, F + bp * MB_WORDS, Fe + bp * MB_S);
}

constexpr size_t mz_band_smem() {
  return (size_t)(2 * MB_WORDS + 2 * MB_S + MXW * 2 * 16) * 4 +
         (size_t)MXW * 16 * MB_XLD * sizeof(double);
}

// CTA = (full block blockIdx.x, 64 vectors), a warp per 16 vectors.
__global__ void __launch_bounds__(32 * MXW, 4)
    k_mz_band(const double *__restrict__ x, const double *out, double *__restrict__ y,
              const unsigned *__restrict__ F, const int *__restrict__ Fe, Geo g) {
  extern __shared__ __align__(16) unsigned char mz_smem[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
  unsigned *sP = reinterpret_cast<unsigned *>(mz_smem);  // both parities' fragments
  int *sE = reinterpret_cast<int *>(sP + 2 * MB_WORDS);   // their row exponents
  int *Es = sE + 2 * MB_S + wid * 2 * 16;                 // [parity][16] column exponents
  double *X = reinterpret_cast<double *>(sE + 2 * MB_S + MXW * 2 * 16) + wid * 16 * MB_XLD;
  const long long b = blockIdx.x;
  oz_load_frag(sP, F + b * 2 * MB_WORDS, 2 * MB_WORDS, sE, Fe + b * 2 * MB_S, 2 * MB_S);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  // tiles of 16 vectors blockIdx.y MXW + wid, + gridDim.y MXW, ...
  for (long long tile = (long long)blockIdx.y * MXW + wid; tile * 16 < g.count;
       tile += (long long)gridDim.y * MXW) {
    const long long v0 = tile * 16;
    const int nv = (int)min(16LL, g.count - v0);
    for (int e = lane; e < 16 * 4 * MB_S; e += 32) {
      const int r = e / (4 * MB_S), m = e - r * (4 * MB_S);
      const bool ok = r < nv;
      l2c_oz::cp_async8(X + r * MB_XLD + m, ok ? x + (v0 + r) * g.N + b * g.h + m : x, ok ? 8 : 0);
    }
    l2c_oz::cp_commit();
    l2c_oz::cp_wait0();
    __syncwarp();
    l2c_oz::stage_fix<2 * MB_S>(X, MB_XLD, 2, 2 * MB_S, Es);
    l2c_oz::stage_fix<2 * MB_S>(X + 1, MB_XLD, 2, 2 * MB_S, Es + 16);
    const long long *Ys = reinterpret_cast<const long long *>(X);
#pragma unroll 1
    for (int p = 0; p < 2; p++) {
      float acc[l2c_oz::NDIAG][MB_NT][4];
      l2c_oz::mma_tile<MB_NT, MB_KC>(sP + p * MB_WORDS, Ys + p, MB_XLD, 2, acc);
      double val[MB_NT][4];
#pragma unroll
      for (int nt = 0; nt < MB_NT; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int ip = 8 * nt + 2 * t4 + (e & 1), r = gq + 8 * (e >> 1);
          val[nt][e] = l2c_oz::to_double(l2c_oz::combine<MB_NT>(acc, nt, e),
                                         sE[p * MB_S + ip] + Es[p * 16 + r] - 52);
        }
      // the sums over this parity's consumed words (the other parity's are the
      // odd / even places, not written here)
      __syncwarp();
#pragma unroll
      for (int nt = 0; nt < MB_NT; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int ip = 8 * nt + 2 * t4 + (e & 1), r = gq + 8 * (e >> 1);
          X[r * MB_XLD + 2 * ip + p] = val[nt][e];
        }
    }
    __syncwarp();
    // y = out_in + band, a row of h outputs per vector
    for (int e = lane; e < 16 * 2 * MB_S; e += 32) {
      const int r = e / (2 * MB_S), i = e - r * (2 * MB_S);
      if (r < nv) {
        const long long v = v0 + r, j = b * g.h + i;
        y[v * g.N + j] = out[v * g.dist + j * g.stride] + X[r * MB_XLD + i];
      }
    }
    __syncwarp();  // the next tile's copies reuse X
  }
}

// The same band at s = 32: per (block, parity) 32 output rows x 64 terms as
// four 16 x 32 pieces (output half hf, term half kh), each with its own row
// scales, and each vector's window normalised per term half: the weights of a
// row fall off along it, so scaling the far half apart keeps its precision
// (one 64-term scale per row gave 1.1e-14).  The two halves' products are
// rounded once each and added in FP64.  A CTA per (block, parity, 64 vectors),
// so that one parity's fragments (24 KB) and its warps' windows fit three CTAs
// per SM; a warp stages its 16 vectors' 64 same-parity values contiguously.
constexpr int MB2_S = 32;
constexpr int MB2_KC = MB2_S / 8;              // 32 terms per piece
constexpr int MB2_WORDS = oz_words(2, MB2_KC);  // one 16 x 32 piece
constexpr int MB2_XLD = 2 * MB2_S + 1;

// Plan time: piece (hf, kh) of (block b, parity p) at F[((bp 2 + hf) 2 + kh)
// MB2_WORDS ..], its row exponents at Fe[((bp 2 + hf) 2 + kh) 16 ..], bp = 2 b
// + p.  One thread per (block, parity, row, term half).
__global__ void k_oz_pack_band2(const double *__restrict__ a, const double *__restrict__ an,
                                const double *__restrict__ dn, Geo g, int c2l,
                                unsigned *__restrict__ F, int *__restrict__ Fe) {
  const long long n = (g.nL - 1) * 2 * MB2_S * 2;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int kh = (int)(idx & 1);
  const long long r2 = idx >> 1, bp = r2 / MB2_S;
  const int ip = (int)(r2 - bp * MB2_S), hf = ip >> 4;
  const long long b = bp >> 1, p = bp & 1, j = b * g.h + 2 * ip + p;
  const long long piece = (bp * 2 + hf) * 2 + kh;
  oz_pack_row(
      [&](int k) {
        const int mp = 32 * kh + k;
        return mp >= ip ? near_weight(c2l, mp - ip, j, a, an, dn) : 0.0;
      },
      true, ip & 15, 32, 2, MB2_KC, F + piece * MB2_WORDS, Fe + piece * 16);
}

constexpr size_t mz_band2_smem() {
  return (size_t)(4 * MB2_WORDS + 4 * 16 + MXW * 2 * 16) * 4 +
         (size_t)MXW * 16 * MB2_XLD * sizeof(double);
}

// CTA = (full block blockIdx.x, parity blockIdx.y & 1, 64 vectors from
// 64 (blockIdx.y >> 1)), a warp per 16 vectors.
__global__ void __launch_bounds__(32 * MXW, 3)
    k_mz_band2(const double *__restrict__ x, const double *out, double *__restrict__ y,
               const unsigned *__restrict__ F, const int *__restrict__ Fe, Geo g) {
  extern __shared__ __align__(16) unsigned char mz_smem[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
  unsigned *sP = reinterpret_cast<unsigned *>(mz_smem);  // the parity's four pieces
  int *sE = reinterpret_cast<int *>(sP + 4 * MB2_WORDS);  // their row exponents
  int *Es = sE + 4 * 16 + wid * 2 * 16;                   // [term half][16] column exponents
  double *X = reinterpret_cast<double *>(sE + 4 * 16 + MXW * 2 * 16) + wid * 16 * MB2_XLD;
  const long long b = blockIdx.x;
  const int p = (int)(blockIdx.y & 1);
  const long long bp = b * 2 + p;
  oz_load_frag(sP, F + bp * 4 * MB2_WORDS, 4 * MB2_WORDS, sE, Fe + bp * 4 * 16, 4 * 16);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  const long long v0 = ((long long)(blockIdx.y >> 1) * MXW + wid) * 16;
  if (v0 >= g.count) return;
  const int nv = (int)min(16LL, g.count - v0);
  for (int e = lane; e < 16 * 2 * MB2_S; e += 32) {  // x[v][b h + 2 m' + p], m' < 2s
    const int r = e / (2 * MB2_S), m = e - r * (2 * MB2_S);
    const bool ok = r < nv;
    l2c_oz::cp_async8(X + r * MB2_XLD + m, ok ? x + (v0 + r) * g.N + b * g.h + 2 * m + p : x,
                      ok ? 8 : 0);
  }
  l2c_oz::cp_commit();
  l2c_oz::cp_wait0();
  __syncwarp();
  l2c_oz::stage_fix<32>(X, MB2_XLD, 1, 32, Es);            // terms 0 .. 31
  l2c_oz::stage_fix<32>(X + 32, MB2_XLD, 1, 32, Es + 16);  // terms 32 .. 63
  const long long *Ys = reinterpret_cast<const long long *>(X);
  double val[2][2][4];
#pragma unroll 1
  for (int hf = 0; hf < 2; hf++) {
#pragma unroll
    for (int nt = 0; nt < 2; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) val[hf][nt][e] = 0.0;
#pragma unroll 1
    for (int kh = 0; kh < 2; kh++) {
      const int pc = hf * 2 + kh;
      long long T[2][4];
      oz_tile_T<2, MB2_KC>(sP + pc * MB2_WORDS, Ys + 32 * kh, MB2_XLD, 1, T);
#pragma unroll
      for (int nt = 0; nt < 2; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int ipl = 8 * nt + 2 * t4 + (e & 1), r = gq + 8 * (e >> 1);
          val[hf][nt][e] +=
              l2c_oz::to_double(T[nt][e], sE[pc * 16 + ipl] + Es[16 * kh + r] - 52);
        }
    }
  }
  __syncwarp();  // every lane is done with the staged words
#pragma unroll
  for (int hf = 0; hf < 2; hf++)
#pragma unroll
    for (int nt = 0; nt < 2; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int ip = 16 * hf + 8 * nt + 2 * t4 + (e & 1), r = gq + 8 * (e >> 1);
        X[r * MB2_XLD + ip] = val[hf][nt][e];
      }
  __syncwarp();
  // y = out_in + band at this parity's outputs j = b h + 2 i' + p
  for (int e = lane; e < 16 * MB2_S; e += 32) {
    const int r = e / MB2_S, i = e - r * MB2_S;
    if (r < nv) {
      const long long v = v0 + r, j = b * g.h + 2 * i + p;
      y[v * g.N + j] = out[v * g.dist + j * g.stride] + X[r * MB2_XLD + i];
    }
  }
}

// The outputs of the last (ragged) block, j >= (nL - 1) h: k_near's FP64 sums.
__global__ void k_mz_band_last(const double *__restrict__ x, const double *out,
                               double *__restrict__ y, const double *__restrict__ a,
                               const double *__restrict__ an, const double *__restrict__ dn,
                               Geo g, int c2l) {
  const long long jlast = (g.nL - 1) * g.h, ntail = g.N - jlast;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (ntail <= 0 || idx >= g.count * ntail) return;
  const long long v = idx / ntail, j = jlast + (idx - v * ntail);
  double res[1];
  near_sums<1>(x + v * g.N + j, g.N, a, an, dn, nullptr, g, c2l, j, res);
  y[v * g.N + j] = out[v * g.dist + j * g.stride] + res[0];
}


// Column format <-> doubles, in place, one thread per 18-coefficient column
// (for the FP64 far-field kernel of single vectors).
__global__ void k_oz_cols_to_double(long long *V, const int *__restrict__ E, long long ncol) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;  // one element
  if (idx >= ncol * M) return;
  const long long t = V[idx];
  reinterpret_cast<double *>(V)[idx] = l2c_oz::to_double(t, E[idx / M] - l2c_oz::VBITS);
}

// 16 columns per CTA of 16 * 18 threads: coalesced loads, one exponent per column.
constexpr int OZ_CONV_COLS = 16;
__global__ void __launch_bounds__(OZ_CONV_COLS * M)
    k_oz_cols_from_double(double *D, int *__restrict__ E, long long ncol) {
  __shared__ int ex[OZ_CONV_COLS * M];
  __shared__ int ecol[OZ_CONV_COLS];
  const long long idx = blockIdx.x * (long long)(OZ_CONV_COLS * M) + threadIdx.x;
  const bool live = idx < ncol * M;
  const double d = live ? D[idx] : 0.0;
  ex[threadIdx.x] = l2c_oz::exp_bound(d);
  __syncthreads();
  if (threadIdx.x < OZ_CONV_COLS) {
    int e = l2c_oz::EXP_ZERO;
    for (int k = 0; k < M; k++) e = max(e, ex[threadIdx.x * M + k]);
    ecol[threadIdx.x] = e;
    const long long col = blockIdx.x * (long long)OZ_CONV_COLS + threadIdx.x;
    if (col < ncol) E[col] = e;
  }
  __syncthreads();
  if (!live) return;
  // |d| < 2^e: V = trunc(d 2^(VBITS - e)), |V| < 2^VBITS
  const int e = ecol[threadIdx.x / M];
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int exb = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = e - l2c_oz::VBITS + 1075 - exb;  // >= -(VBITS - 53)
  unsigned long long q = sh >= 0 ? m >> (sh < 63 ? sh : 63) : m << ((-sh) & 63);
  q = exb == 0 ? 0ull : q;
  reinterpret_cast<long long *>(D)[idx] = (b >> 63) ? -(long long)q : (long long)q;
}

// ---------------------------------------------------------------------------
// Plan
// ---------------------------------------------------------------------------
struct l2c_gpu_plan;
namespace {
struct PhaseScope;
}

// Launch choices of one call shape.  The autotuner searches all but npair;
// none of those changes results: every setting gives the same bits.
//   overlap  : the band on a second stream beside the far-field chain (0/1)
//   pdl      : programmatic dependent launch flags (1 chain, 2 band, 4 the
//              first chain kernel after the band on the same stream)
//   prio     : the chain's kernels at the device's greatest priority (0/1)
//   nthreads : band CTA size while it overlaps (128/256)
//   nvb      : band vectors per thread while it overlaps (1, 2, 4, 8)
//   npair    : band kernel forming outputs in pairs (0/1; not searched: the
//              unpaired kernel splits each sum into even and odd k chains, so
//              the two round differently)
//   nctas    : band grid cap while it overlaps (0: none)
//   nbuf     : tile buffers per warp of the mixed-form kernels (1/2)
//   wtab     : band weights from a table in device memory (the reference's
//              precompute; one DFMA per term instead of DMUL + DFMA, the same
//              products): 1 always, 0 never, -1 by size -- batches whose table
//              is no larger than their input (one table serves every vector of
//              the batch; a single vector's is ~1.5 s times the vector), and
//              plans created with precompute
//   fork     : where the band joins the chain's stream order when it overlaps:
//              0 from the start, 1 after leaf-up, 2 after the upward sweep,
//              3 after the far field (it always finishes before leaf-down);
//              -1 the plan's rule (band_fork_for: from the start)
struct TuneCfg {
  int overlap = -1, pdl = -1, prio = -1, nthreads = 128, nvb = 8, npair = -1, nctas = 0,
      nbuf = 1, wtab = -1, fork = -1;
  // the per-level structure of the far-field chain and the band's schedule:
  //   mtop  mixed form: coarsest transfer level in the one top launch (-2: the
  //         plan's rule, levels of at most 64 slots; -1: none)
  //   mtopg mixed form: trees per CTA of that launch (0: the plan's)
  //   tl0   plain form: level of the subtree roots of the transfer kernels
  //         (-1: by the batch size)
  //   bseg  tiled band: blocks per work unit (0: its cost model)
  //   fsplit mixed batches: the far-field blocks of the fsplit finest levels
  //         run on a third stream, each level as soon as the upward sweep has
  //         its moments, beside the coarser levels' latency-bound launches
  //         (-1: the plan's rule)
  //   bthin tiled band at s = 16: the thin variant (one vector per lane, at
  //         most 64 registers, half the shared memory), which leaves room for
  //         more CTAs of the kernels beside it (-1: the plan's rule)
  //   fartc mixed batches: the far-field products on the fifth-generation
  //         tensor cores (k_mz_far_tc, accumulators in tensor memory) instead
  //         of mma.sync (k_mz_far); the same bits (-1: the plan's rule)
  int mtop = -2, mtopg = 0, tl0 = -1, bseg = 0, fsplit = -1, bthin = -1, fartc = -1;
};
// Two configurations are the same when every choice is (TuneCfg holds only
// ints, so its bytes are its fields).
inline bool same_cfg(const TuneCfg &a, const TuneCfg &b) {
  return std::memcmp(&a, &b, sizeof(TuneCfg)) == 0;
}

// A tuned call shape and its choices (dist is 0 for single vectors).
struct TunedShape {
  size_t dir, count, dist, stride;
  TuneCfg cfg;
  double ms, ms_default;  // per call, tuned and with the plan's defaults
  bool from_cache;
};

struct l2c_gpu_plan {
  size_t N = 0, maxs = 0, L = 0, s = 0, Nn = 0, Nb = 0, h = 0, nL = 0, K = 0, slots = 0;
  size_t dirs = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  double *a = nullptr, *an = nullptr, *dn = nullptr;
  double *A[2] = {nullptr, nullptr};
  double *T = nullptr;
  // scratch, grown on demand
  double *x = nullptr, *y = nullptr, *w = nullptr, *c = nullptr;
  size_t cap_vec = 0;
  double *st_in = nullptr, *st_out = nullptr;
  size_t cap_st_in = 0, cap_st_out = 0;
  size_t flops[2] = {0, 0};
  std::mutex mu;
  // second stream for the near-field band, which runs beside the far-field chain
  cudaStream_t stream2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // third stream for the far-field blocks of the finest levels (TuneCfg::fsplit):
  // per split level a fork event (its moments are ready) and a join event
  cudaStream_t stream3 = nullptr;
  cudaEvent_t ev_ff[FAR_SPLIT_MAX] = {}, ev_fj[FAR_SPLIT_MAX] = {};
  int far_split = -1;  // TuneCfg::fsplit
  int band_thin = -1;  // TuneCfg::bthin
  int far_tc = -1;     // TuneCfg::fartc
  int far_cols = 0;    // k_mz_far's columns per CTA (L2C_FAR_COLS=64|128; 0: by the launch's size)
  double *Wnear[2] = {nullptr, nullptr};  // precomputed band weights (optional)
  // dense band weights of the full blocks for k_band_tile (built on first use)
  double *Wtile[2] = {nullptr, nullptr};
  int band_tile = -1;  // batches' band as dense register tiles: -1 when eligible, 0 never
  int near_rows = -1;  // single vectors' band with register windows: -1 by size, 0 never, 1 always
  int sms = 152;       // multiprocessors of the plan's device
  bool precompute = false;  // created with L2C_PLAN_PRECOMPUTE_NEAR
  bool use_w = false;       // this call's band reads Wnear (see TuneCfg::wtab)
  // nodal (Lagrange) form: T holds barycentric interpolation weights, A the
  // kernel samples, and the trees use B0 | B1 (c_lag_B; host copy lagB)
  bool nodal = false;
  double lagB[2 * MM] = {0};
  // mixed precision (L2C_PLAN_MIXED): sliced constant factors
  bool mixed = false;
  // fragment words (l2c_oz::frag_index layout) and row exponents of: T_parity^T
  // (leaf up), [B | B'] (tree up), B^T and B^T' (tree down), T_parity in passes
  // of 16 rows (leaf down), and the far-field blocks (built on the first batched
  // call, per direction)
  unsigned *oz_lu = nullptr, *oz_tu = nullptr, *oz_td = nullptr, *oz_ld = nullptr;
  int *oz_lum = nullptr, *oz_tum = nullptr, *oz_tdm = nullptr;  // producer metadata
  int *oz_lde = nullptr;                                        // leaf-down row exponents
  int oz_kc = 0, oz_npass = 0;  // leaf-up k8 chunks, leaf-down passes
  int oz_ld_ctas = 1;           // resident leaf-down CTAs per SM
  int oz_tree_q = l2c_oz::SLICES;  // digit slices of the transfer matrices that are not zero
  // tile buffers per warp of the mixed-form kernels: 1 (default) leaves room
  // for twice the warps per SM, which hide more of the products' latency than
  // a second buffer does (256 x 16384: 1.155 vs 1.253 ms per L2C + C2L)
  int oz_nbuf = 1;
  bool zero_copy = true;  // page-locked host buffers used in place (L2C_ZERO_COPY=0: staged)
  unsigned *oz_far[2] = {nullptr, nullptr};
  unsigned *oz_far_tc[2] = {nullptr, nullptr};  // the same words in k_mz_far_tc's layout
  // the band of the full blocks on the tensor cores (k_mz_band): fragments and
  // row exponents per direction, built on the first call that uses them
  unsigned *mz_band[2] = {nullptr, nullptr};
  int *mz_bande[2] = {nullptr, nullptr};
  bool mz_band_on = true;  // L2C_MZ_BAND=0: the FP64 tiled band
  int mz_band_tpw = 1;     // k_mz_band's 16-vector tiles per warp (L2C_MZ_BAND_TPW)
  int *oz_farm[2] = {nullptr, nullptr};
  // column exponents of w and c (mixed form: w, c hold column-format integers)
  int *wE = nullptr, *cE = nullptr;
  size_t cap_wE = 0, cap_cE = 0;
  int *bad = nullptr;  // per vector: an Inf or NaN input seen (mixed form)
  bool mz_top = true;  // the coarsest transfer levels in one launch (mz_top_level)
  int mz_top_lvl = -2;  // TuneCfg::mtop
  int tree_l0 = -1;     // TuneCfg::tl0
  int band_bseg = 0;    // TuneCfg::bseg
  int mz_top_g = 2;    // trees per CTA of that launch
  int mz_top_g_base = 2;  // the plan's own (environment)
  // captured launch sequences, keyed by the call's shape and pointers
  struct GraphEntry {
    size_t dir, count, dist, stride;
    const void *in;
    void *out;
    unsigned mode;
    TuneCfg cfg;  // launch choices the graph was captured with
    bool use_w;   // and whether its band read the weight table
    cudaGraphExec_t exec;
    size_t launches;
    size_t last_use;
  };
  std::vector<GraphEntry> graphs;
  size_t use_clock = 0;
  bool use_graphs = true;
  // Scheduling of a call (see sched_for): -1 = by the call's shape, 0/1 forced.
  //  overlap: the band on stream2 beside the far-field chain;
  int overlap = -1;
  unsigned near_ctas = 0;  // band grid cap while it overlaps (0: no cap)
  int near_vb = 8;         // band vectors per thread while it overlaps
  // band CTA size while it overlaps: 128 threads free registers in pieces the
  // chain's CTAs fit (256 x 16384 mixed: 1.079 -> 1.067 ms; plain batches +0.1 %)
  int near_threads = 128;
  int near_pair = -1;    // band in pairs: 1 always, 0 never, -1 by leaf size
  //  pdl: programmatic dependent launch, bit flags: 1 far-field chain kernels,
  //    2 the band, 4 the first chain kernel after the band on the same stream;
  //  chain_prio_mode: the chain's kernels at the device's greatest priority.
  int pdl = -1;
  int chain_prio_mode = -1;
  int band_fork = -1;  // TuneCfg::fork
  int prio_greatest = 0;  // cudaDeviceGetStreamPriorityRange's greatest priority
  // autotuner: the plan's own choices (defaults and environment), the tuned
  // shapes, a configuration forced while one is timed, and the configuration
  // the fields hold (part of every captured graph's key, with use_w)
  TuneCfg base;
  std::vector<TunedShape> tuned;
  const TuneCfg *forced = nullptr;
  TuneCfg cfg_cur;
  bool autotune = false;          // L2C_AUTOTUNE=1: tune each new shape on its first call
  char tune_cache[1024] = {0};    // L2C_AUTOTUNE_CACHE: file of tuned shapes
  bool tune_cache_loaded = false;
  int oz_ld_ctas_nb[3] = {1, 1, 1};  // resident leaf-down CTAs per SM, by tile buffers
  // launch accounting and optional per-phase CUDA-event timing
  size_t launches = 0;
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;                 // recycled events
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  double phase_ms[L2C_NPHASES] = {0};
  size_t phase_launches[L2C_NPHASES] = {0};
};

namespace {

// Reference flop count (the value execute() returns), reproduced term by term,
// including its unsigned wrap-around in directL's last block (leg2cheb.c:507-516).
size_t ref_flops_geo(size_t N, size_t L, size_t s, size_t Nb, size_t dir, bool nodal = false);
size_t ref_flops(const l2c_gpu_plan *p, size_t dir) {
  return ref_flops_geo(p->N, p->L, p->s, p->Nb, dir, p->nodal);
}

// The reference's flop count (execute's return value): transfer steps count
// M^2 per block (modal) or 4 M^2 (nodal, leg2cheb.c:1414, 1462).
size_t ref_flops_geo(size_t N, size_t L_, size_t s_, size_t Nb, size_t dir, bool nodal) {
  struct {
    size_t L, s, Nb;
  } q{L_, s_, Nb}, *p = &q;
  size_t f = 0;
  if (p->L == 0) {
    f = N;
    for (size_t n = (dir == 0 ? 0 : 2); n < N; n += 2) f += 3 * (N - n);
    return f + N;
  }
  const size_t L = p->L, s = p->s, MMs = (size_t)MM, MMt = (nodal ? 4 : 1) * MMs;
  const size_t K = 2 * (((size_t)2 << (L - 1)) - 1);
  size_t far = 4 * K * s * M;
  for (size_t l = 1; l < L; l++) far += (((size_t)2 << l) - 2) * MMt;       // step 2
  far += 3 * p->Nb * 2 * MMs;                                              // step 3
  for (size_t l = 0; l + 1 < L; l++) far += (((size_t)2 << (l + 1)) - 2) * MMt;  // step 4
  f = 2 * far;
  const size_t h = 2 * s, nL = N / h, i0 = (nL - 1) * h;
  size_t band = 0;
  for (size_t n = (dir == 0 ? 0 : 2); n < 4 * s; n += 2) band += 3 * (n < h ? h : 2 * h - n);
  f += (nL - 1) * band;
  if (dir == 0) {
    for (size_t n = 0; 2 * n + i0 < N; n++) f += 3 * (N - (2 * n + i0));
    f += N;
  } else {
    f += 3 * N;
    for (size_t n = 1; n < N - i0; n++) f += (N - (2 * n + i0)) * 3;
    f += 2 * N;
  }
  return f;
}

bool grow(double **ptr, size_t *cap, size_t need) {
  if (need <= *cap) return true;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(ptr, need * sizeof(double));
  if (e != cudaSuccess) {
    set_err("cudaMalloc(%zu bytes) failed: %s", need * sizeof(double), cudaGetErrorString(e));
    *ptr = nullptr;
    return false;
  }
  *cap = need;
  return true;
}

cudaEvent_t take_event(l2c_gpu_plan *p) {
  if (!p->ev_pool.empty()) {
    cudaEvent_t e = p->ev_pool.back();
    p->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// Brackets the launches of one phase: counts them and, when profiling, records
// CUDA events on the plan's stream around them.
struct PhaseScope {
  l2c_gpu_plan *p;
  int phase;
  cudaEvent_t e0 = nullptr;
  cudaStream_t st;
  PhaseScope(l2c_gpu_plan *pl, int ph, size_t nlaunch, cudaStream_t s_ = nullptr)
      : p(pl), phase(ph), st(s_ ? s_ : pl->stream) {
    p->launches += nlaunch;
    p->phase_launches[ph] += nlaunch;
    if (p->profiling) {
      e0 = take_event(p);
      if (e0) cudaEventRecord(e0, st);
    }
  }
  ~PhaseScope() {
    if (!e0) return;
    cudaEvent_t e1 = take_event(p);
    if (!e1) return;
    cudaEventRecord(e1, st);
    p->pending.push_back({phase, {e0, e1}});
  }
};

void collect_profile(l2c_gpu_plan *p) {
  for (auto &pe : p->pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(pe.second.second) == cudaSuccess &&
        cudaEventElapsedTime(&ms, pe.second.first, pe.second.second) == cudaSuccess)
      p->phase_ms[pe.first] += ms;
    p->ev_pool.push_back(pe.second.first);
    p->ev_pool.push_back(pe.second.second);
  }
  p->pending.clear();
}

// Captured graphs hold scratch and staging addresses: drop them whenever any
// of those buffers is reallocated.
void drop_graphs(l2c_gpu_plan *p) {
  for (auto &g : p->graphs) cudaGraphExecDestroy(g.exec);
  p->graphs.clear();
}

bool ensure_scratch(l2c_gpu_plan *p, size_t count) {
  if (count <= p->cap_vec) return true;
  cudaStreamSynchronize(p->stream);
  cudaStreamSynchronize(p->stream2);
  cudaStreamSynchronize(p->stream3);
  drop_graphs(p);
  size_t c0 = p->cap_vec;
  size_t cx = c0 * p->N, cy = cx, cw = c0 * 2 * p->slots * M, cc = cw;
  const size_t need = count;
  if (!grow(&p->x, &cx, need * p->N) || !grow(&p->y, &cy, need * p->N)) return false;
  if (p->L > 0) {
    if (!grow(&p->w, &cw, need * 2 * p->slots * M) || !grow(&p->c, &cc, need * 2 * p->slots * M))
      return false;
    if (p->mixed) {
      // column exponents: ints, sized in doubles for grow()
      const size_t ne = (need * 2 * p->slots + 1) / 2;
      double *we = reinterpret_cast<double *>(p->wE), *ce = reinterpret_cast<double *>(p->cE);
      size_t cwe = p->cap_wE, cce = p->cap_cE;
      const bool ok = grow(&we, &cwe, ne) && grow(&ce, &cce, ne);
      p->wE = reinterpret_cast<int *>(we);
      p->cE = reinterpret_cast<int *>(ce);
      p->cap_wE = cwe;
      p->cap_cE = cce;
      if (!ok) return false;
      if (p->bad) cudaFree(p->bad);
      p->bad = nullptr;
      if (cudaMalloc(&p->bad, need * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        set_err("cudaMalloc of the mixed-form vector flags failed");
        return false;
      }
    }
  }
  p->cap_vec = need;
  return true;
}

// Device address of page-locked host memory that is mapped into the device's
// address space (nullptr otherwise: pageable memory, or not mapped).
void *mapped_host_ptr(const void *ptr) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

bool is_device_ptr(const void *ptr) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
    else prev = -1;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// How a sweep over L levels is split (see k_up_sub): subtree root level l0,
// subtree depth d = L-1-l0, top-kernel start level lt.  Roots per (vector,
// parity) are 2^(l0+2); l0 is chosen so the subtree kernel has about two CTAs
// per SM, d is at most 7 (shared memory), lt at most 4 (one CTA runs the top).
struct TreePlan {
  int l0, d, lt;
  bool staged;  // false: one tiled launch per level
};

TreePlan tree_plan(size_t L, size_t count, int l0_forced = -1) {
  TreePlan t{0, 0, 0, false};
  if (L < 4) return t;
  int l0 = 0;
  while (l0 + 1 < (int)L - 1 && (double)count * 2.0 * (double)(8LL << l0) <= 2.0 * 152) l0++;
  if (l0_forced >= 0) l0 = std::min(l0_forced, (int)L - 2);
  if ((int)L - 1 - l0 > 7) l0 = (int)L - 8;
  t.l0 = l0;
  t.d = (int)L - 1 - l0;
  t.lt = std::min(l0, 4);
  t.staged = t.d >= 1;
  return t;
}

size_t tree_launches(const TreePlan &t, size_t L) {
  if (!t.staged) return L - 1;
  return 1 + (size_t)(t.l0 - t.lt) + (t.lt > 0 ? 1 : 0);
}

size_t sub_smem(int d) { return ((size_t)(2 << d) - 1) * SUB_PAD * sizeof(double); }
size_t top_smem(int lt) { return ((size_t)(8LL << lt) - 4) * SUB_PAD * sizeof(double); }

template <bool NODAL>
cudaError_t sweep_up_t(double *w, const Geo &g, const TreePlan &t, cudaStream_t st,
                       LaunchOpt pdl) {
  if (!t.staged) {
    for (long long l = g.L - 2; l >= 0; l--) {
      const long long np = (long long)slots_at((size_t)l);
      launch_k(pdl, k_tree_up<NODAL>, blocks_for(g.count * 2 * np, TREE_TILE), 32 * M, 0, st, w, g,
               2 * (long long)blocks_before(l), 2 * (long long)blocks_before(l + 1), np);
    }
    return cudaGetLastError();
  }
  const unsigned nsub = (unsigned)(g.count * 2 * (4LL << t.l0));
  launch_k(pdl, k_up_sub<NODAL>, nsub, 32 * M, sub_smem(t.d), st, w, g, (int)t.l0, (int)t.d);
  for (long long l = t.l0 - 1; l >= t.lt; l--) {
    const long long np = (long long)slots_at((size_t)l);
    launch_k(pdl, k_tree_up<NODAL>, blocks_for(g.count * 2 * np, TREE_TILE), 32 * M, 0, st, w, g,
             2 * (long long)blocks_before(l), 2 * (long long)blocks_before(l + 1), np);
  }
  if (t.lt > 0)
    launch_k(pdl, k_up_top<NODAL>, (unsigned)(g.count * 2), 32 * M, top_smem(t.lt), st, w, g, (int)t.lt);
  return cudaGetLastError();
}

cudaError_t sweep_up(double *w, const Geo &g, const TreePlan &t, cudaStream_t st, LaunchOpt pdl,
                     bool nodal) {
  return nodal ? sweep_up_t<true>(w, g, t, st, pdl) : sweep_up_t<false>(w, g, t, st, pdl);
}

template <bool NODAL>
cudaError_t sweep_down_t(double *c, const Geo &g, const TreePlan &t, cudaStream_t st,
                         LaunchOpt pdl) {
  if (!t.staged) {
    for (long long l = 0; l + 1 < g.L; l++) {
      const long long np = (long long)slots_at((size_t)l);
      launch_k(pdl, k_tree_down<NODAL>, blocks_for(g.count * 2 * np, TREE_TILE), 32 * M, 0, st, c, g,
               2 * (long long)blocks_before(l), 2 * (long long)blocks_before(l + 1), np);
    }
    return cudaGetLastError();
  }
  if (t.lt > 0)
    launch_k(pdl, k_down_top<NODAL>, (unsigned)(g.count * 2), 32 * M, top_smem(t.lt), st, c, g, (int)t.lt);
  for (long long l = t.lt; l < t.l0; l++) {
    const long long np = (long long)slots_at((size_t)l);
    launch_k(pdl, k_tree_down<NODAL>, blocks_for(g.count * 2 * np, TREE_TILE), 32 * M, 0, st, c, g,
             2 * (long long)blocks_before(l), 2 * (long long)blocks_before(l + 1), np);
  }
  const unsigned nsub = (unsigned)(g.count * 2 * (4LL << t.l0));
  launch_k(pdl, k_down_sub<NODAL>, nsub, 32 * M, sub_smem(t.d), st, c, g, (int)t.l0, (int)t.d);
  return cudaGetLastError();
}

cudaError_t sweep_down(double *c, const Geo &g, const TreePlan &t, cudaStream_t st, LaunchOpt pdl,
                       bool nodal) {
  return nodal ? sweep_down_t<true>(c, g, t, st, pdl) : sweep_down_t<false>(c, g, t, st, pdl);
}

// Near field for all vectors of a batch: full groups of 8 (4, 2) vectors per
// thread, then the remainder.
cudaError_t launch_near(const double *x, const double *out, double *y, const double *a,
                        const double *an, const double *dn, const double *W, Geo g, int c2l,
                        cudaStream_t st, bool pair, unsigned max_ctas, int max_vb,
                        bool pdl = false, int threads = 256, long long jbeg = 0) {
  long long v = 0;
  while (v < g.count) {
    const long long left = g.count - v;
    int vb = left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
    vb = std::min(vb, max_vb);
    const long long groups = left / vb;
    Geo gg = g;
    gg.count = groups * vb;
    const double *xs = x + v * g.N;
    const double *os = out + v * g.dist;
    double *ys = y + v * g.N;
    if (!pair) {
      unsigned grid = (unsigned)(((g.N - jbeg + threads - 1) / threads) * groups);
      if (max_ctas) grid = std::min(grid, max_ctas);
      auto *kern = vb == 8 ? k_near<8> : vb == 4 ? k_near<4> : vb == 2 ? k_near<2> : k_near<1>;
      launch_k(pdl, kern, grid, threads, 0, st, xs, os, ys, a, an, dn, W, gg, c2l, jbeg);
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      v += groups * vb;
      continue;
    }
    // blocks b < nL-1 in pairs and the last (ragged) block one output per thread
    const long long per_vg = (g.nL - 1) * (g.h / 2) + (g.N - (g.nL - 1) * g.h);
    unsigned grid = (unsigned)((groups * per_vg + threads - 1) / threads);
    if (max_ctas) grid = std::min(grid, max_ctas);
    auto *kern = vb == 8   ? k_near_pair<8>
                 : vb == 4 ? k_near_pair<4>
                 : vb == 2 ? k_near_pair<2>
                           : k_near_pair<1>;
    launch_k(pdl, kern, grid, threads, 0, st, xs, os, ys, a, an, dn, W, gg, c2l);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    v += groups * vb;
  }
  return cudaSuccess;
}

// Whether this call's band runs as k_band_tile (full blocks) + k_near (last block).
bool use_band_tile(const l2c_gpu_plan *p, size_t count) {
  return p->band_tile != 0 && p->L > 0 && band_tile_ok((long long)p->s, (long long)p->nL,
                                                       (long long)count);
}

// Whether a mixed batch's band runs on the tensor cores (k_mz_band): the
// batches whose FP64 band would be dense tiles, at s = 16.
bool use_mz_band(const l2c_gpu_plan *p, size_t count) {
  return p->mixed && p->mz_band_on && (p->s == (size_t)MB_S || p->s == (size_t)MB2_S) &&
         p->nL >= 2 && use_band_tile(p, count);
}

// Whether this call's band runs as k_near_rows (full blocks and, one output
// per thread, the last block): single vectors with enough blocks (any with
// L2C_NEAR_ROWS=1, none with 0), unless the paired kernel is forced
// (L2C_NEAR_PAIR).
bool use_near_rows(const l2c_gpu_plan *p, size_t count) {
  return p->near_rows != 0 && p->near_pair != 1 && p->L > 0 &&
         near_rows_ok((long long)p->s, (long long)p->nL, (long long)count, p->near_rows == 1);
}

// Whether the tiled band takes its thin variant (TuneCfg::bthin; s = 16 only).
// By default in the mixed form, where the chain beside the band is bound by
// integer latency and gains from the registers and shared memory the thin
// band leaves it (256 x 16384, untuned: 0.824 -> 0.768 ms per L2C + C2L); the
// FP64 chain of plain batches needs no more room.  The same sums per output,
// so the same bits.
bool band_tile_thin(const l2c_gpu_plan *p) {
  return p->s == 16 && (p->band_thin >= 0 ? p->band_thin == 1 : p->mixed);
}

// Band of a batch through k_band_tile, one launch (the full blocks; Wt: its
// dense table or nullptr for weights formed on the fly; the last block with
// weights formed on the fly: the same products, so the same bits).  Work units: the
// run of blocks per unit (bseg) is the one whose rounds of units over the grid
// finish first, counting half a block for the extra half window a unit loads.
cudaError_t launch_band_tile(const l2c_gpu_plan *p, const double *x, const double *out,
                             double *y, const double *Wt, Geo g, int c2l, cudaStream_t st,
                             unsigned max_ctas, bool pdl) {
  const bool thin = band_tile_thin(p);
  const long long VCH = 32LL * band_tile_c(g.s, thin);
  const long long nchunk = (g.count + VCH - 1) / VCH, nfull = g.nL - 1;
  const long long grid_cap = max_ctas ? (long long)max_ctas : 2LL * p->sms;
  long long best_seg = 1;
  double best = 1e300;
  for (long long bseg = 1; bseg <= std::min<long long>(nfull, 16); bseg++) {
    const long long units = nchunk * ((nfull + bseg - 1) / bseg);
    const long long grid = std::min(units, grid_cap);
    const double t = (double)((units + grid - 1) / grid) * ((double)bseg + 0.5);
    if (t < best) {
      best = t;
      best_seg = bseg;
    }
  }
  if (p->band_bseg > 0) best_seg = std::min<long long>(p->band_bseg, std::max(nfull, 1LL));
  // the chunks' last-block units first, then the full blocks
  const long long units = nchunk * (1 + (nfull + best_seg - 1) / best_seg);
  const unsigned grid = (unsigned)std::min(units, grid_cap);
  auto *kern = Wt ? band_tile_kernel<true>(g.s, thin) : band_tile_kernel<false>(g.s, thin);
  launch_k(pdl, kern, grid, BT_THREADS, band_tile_smem(g.s, thin), st, x, out, y, Wt,
           (const double *)p->a, (const double *)p->an, (const double *)p->dn, g, c2l, nchunk,
           best_seg);
  return cudaGetLastError();
}

// Pairs pay off when a warp's outputs have very unequal term counts (small
// leaves: one warp spans a whole block).
bool near_pair(const l2c_gpu_plan *p) { return p->near_pair >= 0 ? p->near_pair == 1 : p->s <= 16; }

size_t near_launch_count(size_t count, int max_vb) {
  size_t n = 0, v = 0;
  while (v < count) {
    const size_t left = count - v;
    const size_t vb = std::min<size_t>(left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1, max_vb);
    v += (left / vb) * vb;
    n++;
  }
  return n;
}

Geo make_geo(const l2c_gpu_plan *p, size_t count, size_t dist, size_t stride) {
  Geo g;
  g.N = (long long)p->N;
  g.s = (long long)p->s;
  g.h = (long long)p->h;
  g.nL = (long long)p->nL;
  g.L = (long long)p->L;
  g.K = (long long)p->K;
  g.slots = (long long)p->slots;
  g.leaf_base = p->L > 0 ? 2 * (long long)blocks_before(p->L - 1) : 0;
  g.count = (long long)count;
  g.dist = (long long)dist;
  g.stride = (long long)stride;
  return g;
}

// Far field of the mixed form: leaf, tree and far-field products on tensor
// cores (the far-field blocks only when the batch gives each block at least 8
// right-hand sides; single vectors keep the FP64 block products, on doubles
// converted from and back to the column format in place).
// How one call is scheduled.  The band (FP64-bound, many long CTAs) runs on the
// second stream beside the far-field chain.  When the chain is latency-bound --
// a single vector, whose tree levels hold few items, or any mixed plan, whose
// tensor-core kernels are bound by integer latency -- its kernels also carry
// the device's greatest priority (as band CTAs retire the SMs go to the chain
// first; graph nodes keep the priority) and programmatic dependent launch
// (each kernel's prologue and launch overlap the previous kernel).  Measured,
// L2C + C2L: plain single N = 2^20 1.321 -> 1.177 ms, N = 2^14 0.180 -> 0.135;
// mixed 256 x 16384 1.276 -> 1.080.  Plain batches keep plain launches (their
// chain is throughput-bound: 4096 x 1024 2.27 ms, 2.33 with both).
struct Sched {
  bool ov;       // band on the second stream
  unsigned pdl;  // programmatic dependent launch flags (as l2c_gpu_plan::pdl)
  int prio;      // priority of the chain's kernels (0: the stream's)
};

// The band's fork point when the plan leaves it open (TuneCfg::fork = -1):
// from the start.  Where entering after leaf-up pays depends on the size
// (single vectors, L2C + C2L, ms per step, from the start with chain priority
// / after leaf-up without: N = 2^18 0.374 / 0.450, 2^20 1.110 / 1.081, 2^22
// 4.008 / 4.045), so it is left to the autotuner.
int band_fork_for(const l2c_gpu_plan *p, size_t count) {
  (void)count;
  return p->band_fork >= 0 ? std::min(p->band_fork, 3) : 0;
}

Sched sched_for(const l2c_gpu_plan *p, size_t count) {
  Sched sc;
  sc.ov = p->overlap >= 0 ? p->overlap == 1 : true;
  const bool latency = p->mixed || count == 1;
  sc.pdl = p->pdl >= 0 ? (unsigned)p->pdl : latency ? 1u : 0u;
  // a band that enters after leaf-up (band_fork_for) is the longer stream
  // from then on: the chain beside it takes the SMs it leaves, at its own priority
  const bool prio = p->chain_prio_mode >= 0 ? p->chain_prio_mode == 1
                                            : latency && band_fork_for(p, count) == 0;
  sc.prio = prio && sc.ov ? p->prio_greatest : 0;
  return sc;
}

// The first far-field kernel follows the band on the same stream unless the
// band runs on the second stream.
bool pdl_after_band(const Sched &sc) { return (sc.pdl & (sc.ov ? 1u : 4u)) != 0; }

// Levels from .. to (either order), as a transfer kernel's list; G trees per CTA.
TreeLevels tree_levels(long long from, long long to, int G) {
  TreeLevels T{};
  T.G = G;
  const long long step = to >= from ? 1 : -1;
  for (long long l = from;; l += step) {
    T.lv[T.n++] = TreeLevel{2 * (long long)blocks_before((size_t)l),
                            2 * (long long)blocks_before((size_t)l + 1),
                            (long long)slots_at((size_t)l)};
    if (l == to) break;
  }
  return T;
}

// The coarsest levels 0 .. lt of the mixed form's transfer trees go in one
// launch, a CTA per tree (TOP kernels): those with at most 64 slots per tree,
// i.e. at most one tile per warp (-1: none; L2C_MZ_TOP=0 turns this off).
int mz_top_level(const l2c_gpu_plan *p) {
  if (!p->mz_top || p->L < 2 || p->mz_top_lvl == -1) return -1;
  if (p->mz_top_lvl >= 0) return std::min({p->mz_top_lvl, (int)p->L - 2, TREE_TOP_MAX - 1});
  int lt = -1;
  while (lt + 1 <= (int)p->L - 2 && lt + 1 < TREE_TOP_MAX && slots_at((size_t)lt + 1) <= 64)
    lt++;
  return lt;
}

// Whether a mixed batch's far field runs on the fifth-generation tensor cores
// (TuneCfg::fartc; the plan's rule: mma.sync).
bool far_tc_on(const l2c_gpu_plan *p) { return p->far_tc == 1; }

// The mixed form's far-field split (TuneCfg::fsplit): the far-field blocks
// of levels L - n .. L - 1 run on the plan's third stream, level by level as
// the upward sweep writes their moments, beside the coarser levels' transfer
// launches, which are latency-bound and leave most of the GPU idle.  The
// finest two levels hold three quarters of the blocks.  Only levels finer than
// the top launch split (their moments come from a launch of their own), never
// level 0; batches with the tensor-core far field only; none while profiling
// per phase (the phases stay in stream order).  The same bits either way.
int mz_far_split(const l2c_gpu_plan *p, const Geo &g, int lt) {
  if (p->profiling || g.count < 4 || g.L < 3) return 0;
  const int n = p->far_split >= 0 ? p->far_split : 3;
  const int lo = std::max(lt + 1, 1);  // the coarsest level that may split
  return std::max(0, std::min({n, (int)g.L - lo, FAR_SPLIT_MAX}));
}

template <int KC>
void mz_leaf_up_launch(l2c_gpu_plan *p, const double *x, const Geo &g, cudaStream_t st,
                       LaunchOpt pdl) {
  const long long tiles = g.count * ((g.K + 15) / 16);
  const unsigned grid = (unsigned)std::min<long long>((tiles + MXW - 1) / MXW, 152 * 4);
  launch_k(pdl, p->oz_nbuf == 1 ? k_mz_leaf_up<KC, 1> : k_mz_leaf_up<KC, 2>, grid, 32 * MXW,
           mz_leaf_up_smem(KC, p->oz_nbuf), st, x,
           reinterpret_cast<long long *>(p->w), p->wE, (const unsigned *)p->oz_lu,
           (const int *)p->oz_lum, g, p->bad);
}

bool launch_mixed_far(l2c_gpu_plan *p, const double *x, double *out, size_t dir, const Geo &g,
                      cudaStream_t st, const Sched &sc, const std::function<bool(int)> &band) {
  const bool ov = sc.ov;
  const int c2l = dir == 1;
  if (!band(0)) return false;
  long long *w = reinterpret_cast<long long *>(p->w), *c = reinterpret_cast<long long *>(p->c);
  const LaunchOpt chain(sc.pdl & 1, sc.prio);
  if (cudaMemsetAsync(p->bad, 0, (size_t)g.count * sizeof(int), st) != cudaSuccess) return false;
  {
    PhaseScope ps(p, L2C_PHASE_LEAF_UP, 1);
    const LaunchOpt pdl(pdl_after_band(sc), sc.prio);
    switch (p->oz_kc) {
      case 1: mz_leaf_up_launch<1>(p, x, g, st, pdl); break;
      case 2: mz_leaf_up_launch<2>(p, x, g, st, pdl); break;
      case 3: mz_leaf_up_launch<3>(p, x, g, st, pdl); break;
      case 4: mz_leaf_up_launch<4>(p, x, g, st, pdl); break;
      case 5: mz_leaf_up_launch<5>(p, x, g, st, pdl); break;
      case 6: mz_leaf_up_launch<6>(p, x, g, st, pdl); break;
      case 7: mz_leaf_up_launch<7>(p, x, g, st, pdl); break;
      default: mz_leaf_up_launch<8>(p, x, g, st, pdl); break;
    }
    if (cudaGetLastError() != cudaSuccess) return false;
  }
  if (!band(1)) return false;
  const int lt = mz_top_level(p);
  const bool tc = g.count >= 4 && p->oz_far[dir] != nullptr;
  // far-field blocks gb0 .. gb1 - 1 (tensor-core form)
  auto far_launch = [&](long long gb0, long long gb1, cudaStream_t s, LaunchOpt o) {
    if (gb1 <= gb0) return;
    if (far_tc_on(p)) {
      const dim3 grid((unsigned)(gb1 - gb0), (unsigned)((2 * g.count + FTC_COLS - 1) / FTC_COLS));
      launch_k(o, k_mz_far_tc, grid, FTC_THREADS, ftc_smem(), s, (const long long *)w,
               (const int *)p->wE, c, p->cE, (const unsigned *)p->oz_far_tc[dir],
               (const int *)p->oz_farm[dir], g, gb0, p->bad);
      return;
    }
    // columns per CTA: one tile per warp when the launch would not fill
    // the GPU once with two (its latency is then one tile's), else two
    const long long nc2 = (2 * g.count + OZ_FAR_COLS - 1) / OZ_FAR_COLS;
    const int cols = p->far_cols > 0 ? p->far_cols
                     : (gb1 - gb0) * nc2 <= 4LL * p->sms ? OZ_FAR_COLS / 2 : OZ_FAR_COLS;
    const dim3 grid((unsigned)(gb1 - gb0), (unsigned)((2 * g.count + cols - 1) / cols));
    launch_k(o, p->oz_nbuf == 1 ? k_mz_far<1> : k_mz_far<2>, grid, 32 * MXW,
             oz_far_smem(p->oz_nbuf), s, (const long long *)w, (const int *)p->wE, c, p->cE,
             (const unsigned *)p->oz_far[dir], (const int *)p->oz_farm[dir], g, gb0, cols);
  };
  // The finest nsplit levels' far field on stream3 (mz_far_split): level l
  // (split index L - 1 - l) forks once the chain has its moments and joins
  // before the first transfer launch that adds into its far field.
  const int nsplit = tc ? mz_far_split(p, g, lt) : 0;
  auto split_index = [&](long long l) { return (int)(g.L - 1 - l); };
  auto fork_far = [&](long long l) -> bool {
    const int k = split_index(l);
    if (k < 0 || k >= nsplit) return true;
    PhaseScope ps(p, L2C_PHASE_FAR, 1, p->stream3);
    if (cudaEventRecord(p->ev_ff[k], st) != cudaSuccess ||
        cudaStreamWaitEvent(p->stream3, p->ev_ff[k], 0) != cudaSuccess)
      return false;
    far_launch((long long)blocks_before((size_t)l), (long long)blocks_before((size_t)l + 1),
               p->stream3, LaunchOpt(false, sc.prio));
    return cudaGetLastError() == cudaSuccess &&
           cudaEventRecord(p->ev_fj[k], p->stream3) == cudaSuccess;
  };
  // joins the split levels a .. b into the chain's stream; joined: any did
  auto join_far = [&](long long a, long long b, bool &joined) -> bool {
    joined = false;
    for (long long l = a; l <= b; l++) {
      const int k = split_index(l);
      if (k < 0 || k >= nsplit) continue;
      if (cudaStreamWaitEvent(st, p->ev_fj[k], 0) != cudaSuccess) return false;
      joined = true;
    }
    return true;
  };
  if (!fork_far(g.L - 1)) return false;
  {
    PhaseScope ps(p, L2C_PHASE_TREE_UP, (size_t)(g.L - 2 - lt + (lt >= 0 ? 1 : 0)));
    const bool q2 = p->oz_tree_q == 2, nb1 = p->oz_nbuf == 1;
    auto *kup = q2 ? (nb1 ? k_mz_tree_up<2, 1> : k_mz_tree_up<2, 2>)
                   : (nb1 ? k_mz_tree_up<l2c_oz::SLICES, 1> : k_mz_tree_up<l2c_oz::SLICES, 2>);
    for (long long l = g.L - 2; l > lt; l--) {
      const long long tiles = (g.count * 2 * (long long)slots_at((size_t)l) + 15) / 16;
      const unsigned grid = (unsigned)std::min<long long>((tiles + MXW - 1) / MXW, 152 * 4);
      launch_k(chain, kup, grid, 32 * MXW, oz_tree_up_smem(p->oz_tree_q, p->oz_nbuf), st, w,
               p->wE, (const unsigned *)p->oz_tu, (const int *)p->oz_tum, g,
               tree_levels(l, l, 1));
      if (!fork_far(l)) return false;
    }
    if (lt >= 0)  // the top levels lt .. 0, each CTA mz_top_g trees
      launch_k(chain, q2 ? k_mz_tree_up<2, 1, true> : k_mz_tree_up<l2c_oz::SLICES, 1, true>,
               (unsigned)((g.count * 2 + p->mz_top_g - 1) / p->mz_top_g), 32 * MXW,
               oz_tree_up_smem(p->oz_tree_q, 1), st, w, p->wE, (const unsigned *)p->oz_tu,
               (const int *)p->oz_tum, g, tree_levels(lt, 0, p->mz_top_g));
    if (cudaGetLastError() != cudaSuccess) return false;
  }
  if (!band(2)) return false;
  {
    PhaseScope ps(p, L2C_PHASE_FAR, tc ? 1 : 3);
    if (tc) {
      // the levels that did not split
      far_launch(0, (long long)blocks_before((size_t)(g.L - nsplit)), st, chain);
    } else {
      const long long ncol = g.count * 2 * g.slots, n = g.count * (long long)p->Nb * M;
      k_oz_cols_to_double<<<blocks_for(ncol * M, 256), 256, 0, st>>>(w, p->wE, ncol);
      k_far<<<blocks_for(n, 256), 256, 0, st>>>(p->A[dir], p->w, p->c, g, (long long)p->Nb);
      k_oz_cols_from_double<<<blocks_for(ncol, OZ_CONV_COLS), OZ_CONV_COLS * M, 0, st>>>(
          p->c, p->cE, ncol);
    }
    if (cudaGetLastError() != cudaSuccess) return false;
  }
  if (!band(3)) return false;
  {
    PhaseScope ps(p, L2C_PHASE_TREE_DOWN, (size_t)(g.L - 2 - lt + (lt >= 0 ? 1 : 0)));
    const bool q2 = p->oz_tree_q == 2, nb1 = p->oz_nbuf == 1;
    auto *kdown = q2 ? (nb1 ? k_mz_tree_down<2, 1> : k_mz_tree_down<2, 2>)
                     : (nb1 ? k_mz_tree_down<l2c_oz::SLICES, 1>
                            : k_mz_tree_down<l2c_oz::SLICES, 2>);
    // a launch right after a join: a plain launch (full dependency)
    bool joined = false;
    if (lt >= 0) {  // the top levels 0 .. lt, each CTA mz_top_g trees
      if (!join_far(0, lt + 1, joined)) return false;
      launch_k(joined ? LaunchOpt(false, sc.prio) : chain,
               q2 ? k_mz_tree_down<2, 1, true> : k_mz_tree_down<l2c_oz::SLICES, 1, true>,
               (unsigned)((g.count * 2 + p->mz_top_g - 1) / p->mz_top_g), 32 * MXW,
               oz_tree_down_smem(p->oz_tree_q, 1), st, c, p->cE, (const unsigned *)p->oz_td,
               (const int *)p->oz_tdm, g, tree_levels(0, lt, p->mz_top_g));
    }
    for (long long l = lt + 1; l + 1 < g.L; l++) {
      if (!join_far(l + 1, l + 1, joined)) return false;
      const long long tiles = (g.count * 2 * (long long)slots_at((size_t)l) + 15) / 16;
      const unsigned grid = (unsigned)std::min<long long>((tiles + MXW - 1) / MXW, 152 * 4);
      launch_k(joined ? LaunchOpt(false, sc.prio) : chain, kdown, grid, 32 * MXW,
               oz_tree_down_smem(p->oz_tree_q, p->oz_nbuf), st, c, p->cE,
               (const unsigned *)p->oz_td, (const int *)p->oz_tdm, g, tree_levels(l, l, 1));
    }
    if (cudaGetLastError() != cudaSuccess) return false;
  }
  if (ov && cudaStreamWaitEvent(st, p->ev_join, 0) != cudaSuccess) return false;
  {
    PhaseScope ps(p, L2C_PHASE_LEAF_DOWN, 1);
    const long long tiles = g.count * ((g.K + 15) / 16);
    const unsigned grid =
        (unsigned)std::min<long long>((tiles + MXW - 1) / MXW, 152LL * p->oz_ld_ctas);
    // after the join with the band's stream: a plain launch (full dependency)
    launch_k((sc.pdl & 1) && !ov, p->oz_nbuf == 1 ? k_mz_leaf_down<1> : k_mz_leaf_down<2>,
             grid, 32 * MXW, mz_leaf_down_smem(p->oz_npass, p->oz_nbuf, g.h), st,
             (const long long *)c, (const int *)p->cE, (const double *)p->y, out,
             (const unsigned *)p->oz_ld, (const int *)p->oz_lde, g, c2l, p->oz_npass,
             (const int *)p->bad);
    if (cudaGetLastError() != cudaSuccess) return false;
  }
  return true;
}

// Far-field block fragments of the mixed form, built on the first batched call.
bool ensure_mixed_far(l2c_gpu_plan *p, size_t dir) {
  if (p->oz_far[dir]) return true;
  const size_t nb = p->Nb;
  if (cudaMalloc(&p->oz_far[dir], nb * OZ_FAR_WORDS * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&p->oz_farm[dir], nb * 2 * OZ_META * sizeof(int)) != cudaSuccess) {
    set_err("cudaMalloc of the mixed-form far-field fragments failed");
    return false;
  }
  k_oz_pack_far<<<blocks_for((long long)(nb * 2), 128), 128, 0, p->stream>>>(
      p->A[dir], (long long)nb, p->oz_far[dir], p->oz_farm[dir]);
  return cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(p->stream) == cudaSuccess;
}

// The band fragments of one direction for k_mz_band, built on the first call
// that uses them (outside any capture).
bool ensure_mz_band(l2c_gpu_plan *p, size_t dir) {
  if (p->mz_band[dir]) return true;
  const long long nbp = ((long long)p->nL - 1) * 2;
  const bool s32 = p->s == (size_t)MB2_S;
  const size_t words = s32 ? 4 * (size_t)MB2_WORDS : (size_t)MB_WORDS;
  const size_t rows = s32 ? 4 * 16 : (size_t)MB_S;  // row exponents per (block, parity)
  if (cudaMalloc(&p->mz_band[dir], (size_t)nbp * words * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&p->mz_bande[dir], (size_t)nbp * rows * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    set_err("cudaMalloc of the tensor-core band fragments failed");
    return false;
  }
  Geo g = make_geo(p, 1, p->N, 1);
  if (s32)
    k_oz_pack_band2<<<blocks_for(nbp * MB2_S * 2, 128), 128, 0, p->stream>>>(
        p->a, p->an, p->dn, g, (int)dir, p->mz_band[dir], p->mz_bande[dir]);
  else
    k_oz_pack_band<<<blocks_for(nbp * MB_S, 128), 128, 0, p->stream>>>(
        p->a, p->an, p->dn, g, (int)dir, p->mz_band[dir], p->mz_bande[dir]);
  return cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(p->stream) == cudaSuccess;
}

// The far-field fragments in k_mz_far_tc's layout, built on the first call
// that uses that kernel (after ensure_mixed_far).
bool ensure_mixed_far_tc(l2c_gpu_plan *p, size_t dir) {
  if (p->oz_far_tc[dir]) return true;
  const long long nb = (long long)p->Nb;
  if (cudaMalloc(&p->oz_far_tc[dir], (size_t)nb * FTC_B_WORDS * sizeof(unsigned)) !=
      cudaSuccess) {
    cudaGetLastError();
    p->oz_far_tc[dir] = nullptr;
    set_err("cudaMalloc of the tensor-memory far-field fragments failed");
    return false;
  }
  k_oz_pack_far_tc<<<blocks_for(nb * FTC_B_WORDS, 256), 256, 0, p->stream>>>(
      p->oz_far[dir], nb, p->oz_far_tc[dir]);
  return cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(p->stream) == cudaSuccess;
}

// The launch sequence of one batch on device pointers (scratch already sized).
// Near field on stream2 beside the far-field chain on stream; joined before the
// final leaf-down kernel.
size_t launch_all(l2c_gpu_plan *p, const double *in, double *out, size_t dir, size_t count,
                  size_t dist, size_t stride, bool near_only, bool input_ready,
                  bool in_host = false) {
  cudaStream_t st = p->stream, st2 = p->stream2;
  const int c2l = dir == 1;
  Geo g = make_geo(p, count, dist, stride);
  const long long total = g.count * g.N;
  if (p->L == 0) {
    // Vectors whose windows overlap (dist < (N-1) stride + 1, e.g. the columns
    // of a row-major array): each vector's contiguous zeroing of [0, N) and
    // contiguous L2C read reach the other vectors' elements, so the vectors run
    // one after another, as the reference's execute2D calls execute() column
    // by column (leg2cheb.c:1270-1274).  Within one vector the zeroed elements
    // and the accumulated ones (i stride >= N) are distinct.
    if (count > 1 && stride > 1 && dist < (p->N - 1) * stride + 1) {
      PhaseScope ps(p, L2C_PHASE_DIRECT, count);
      Geo g1 = g;
      g1.count = 1;
      for (size_t v = 0; v < count; v++)
        k_direct<<<blocks_for(g.N, 256), 256, 0, st>>>(in + v * dist, out + v * dist, p->a,
                                                       p->an, p->dn, g1, c2l);
      CK(cudaGetLastError());
      return 1;
    }
    PhaseScope ps(p, L2C_PHASE_DIRECT, 1);
    k_direct<<<blocks_for(total, 256), 256, 0, st>>>(in, out, p->a, p->an, p->dn, g, c2l);
    CK(cudaGetLastError());
    return 1;
  }
  // contiguous (and for C2L premultiplied) copy of the input
  const double *x = in;
  // (input in host memory: read once, here, not by every band term)
  if (!input_ready && (in_host || c2l || stride != 1 || (count > 1 && dist != p->N))) {
    PhaseScope ps(p, L2C_PHASE_GATHER, 1);
    k_gather<<<blocks_for(total, 256), 256, 0, st>>>(in, p->x, g, c2l);
    CK(cudaGetLastError());
    x = p->x;
  }
  const bool dense_w = use_band_tile(p, count) || use_near_rows(p, count);
  const double *W = p->use_w && !dense_w ? p->Wnear[dir] : nullptr;
  const double *Wt = p->use_w && dense_w ? p->Wtile[dir] : nullptr;
  if (near_only) {
    {
      PhaseScope ps(p, L2C_PHASE_NEAR, near_launch_count(count, 8));
      CK(launch_near(x, out, p->y, p->a, p->an, p->dn, W, g, c2l, st, near_pair(p), 0, 8));
    }
    Geo g0 = g;
    g0.K = 0;
    PhaseScope ps(p, L2C_PHASE_LEAF_DOWN, 1);
    k_leaf_down<<<blocks_for(total, 256), 256, 0, st>>>(p->c, p->T, p->y, out, g0, c2l);
    CK(cudaGetLastError());
    return 1;
  }
  // The band on the second stream beside the far-field chain (sched_for),
  // entering it at fork point band_fork of the chain (TuneCfg::fork); it
  // always finishes before leaf-down.  Without the second stream it runs
  // first, on the chain's stream.
  const Sched sc = sched_for(p, count);
  const bool ov = sc.ov;
  cudaStream_t stn = ov ? st2 : st;
  const int fork = ov ? band_fork_for(p, count) : 0;
  bool band_done = false;
  auto band = [&](int pos) -> bool {
    if (band_done || pos < fork) return true;
    band_done = true;
    if (ov && (cudaEventRecord(p->ev_fork, st) != cudaSuccess ||
               cudaStreamWaitEvent(st2, p->ev_fork, 0) != cudaSuccess))
      return false;
    if (use_mz_band(p, count)) {
      // the full blocks on the tensor cores, the last block in FP64
      PhaseScope ps(p, L2C_PHASE_NEAR, 2, stn);
      if (g.s == MB2_S)
        launch_k((sc.pdl & 2) && !ov, k_mz_band2,
                 dim3((unsigned)(g.nL - 1), 2 * (unsigned)((g.count + 16 * MXW - 1) / (16 * MXW))),
                 32 * MXW, mz_band2_smem(), stn, x, (const double *)out, p->y,
                 (const unsigned *)p->mz_band[dir], (const int *)p->mz_bande[dir], g);
      else
        launch_k((sc.pdl & 2) && !ov, k_mz_band,
                 dim3((unsigned)(g.nL - 1), (unsigned)((g.count + 16 * MXW * p->mz_band_tpw - 1) /
                                                       (16 * MXW * p->mz_band_tpw))),
                 32 * MXW, mz_band_smem(), stn, x, (const double *)out, p->y,
                 (const unsigned *)p->mz_band[dir], (const int *)p->mz_bande[dir], g);
      const long long ntail = g.N - (g.nL - 1) * g.h;
      k_mz_band_last<<<blocks_for(g.count * ntail, 256), 256, 0, stn>>>(
          x, out, p->y, p->a, p->an, p->dn, g, c2l);
      if (cudaGetLastError() != cudaSuccess) return false;
    } else if (use_band_tile(p, count)) {
      PhaseScope ps(p, L2C_PHASE_NEAR, 1, stn);
      if (launch_band_tile(p, x, out, p->y, p->use_w ? p->Wtile[dir] : nullptr, g, c2l, stn,
                           ov ? p->near_ctas : 0, (sc.pdl & 2) && !ov) != cudaSuccess)
        return false;
    } else if (use_near_rows(p, count)) {
      // full blocks with register windows, the last block per output, one launch
      PhaseScope ps(p, L2C_PHASE_NEAR, 1, stn);
      launch_k((sc.pdl & 2) && !ov, Wt ? k_near_rows<true> : k_near_rows<false>,
               blocks_for(near_rows_items(g), 256), 256, 0, stn, x,
               (const double *)out, p->y, (const double *)p->a, (const double *)p->an,
               (const double *)p->dn, Wt, g, c2l);
      if (cudaGetLastError() != cudaSuccess) return false;
    } else {
      PhaseScope ps(p, L2C_PHASE_NEAR, near_launch_count(count, ov ? p->near_vb : 8), stn);
      if (launch_near(x, out, p->y, p->a, p->an, p->dn, W, g, c2l, stn, near_pair(p),
                      ov ? p->near_ctas : 0, ov ? p->near_vb : 8, (sc.pdl & 2) && !ov,
                      ov ? p->near_threads : 256) != cudaSuccess)
        return false;
    }
    return !ov || cudaEventRecord(p->ev_join, st2) == cudaSuccess;
  };
  if (p->mixed) return launch_mixed_far(p, x, out, dir, g, st, sc, band) ? 1 : 0;
  if (!band(0)) return 0;
  const long long leaf_threads = g.count * g.K * 2 * M;
  {
    PhaseScope ps(p, L2C_PHASE_LEAF_UP, 1);
    launch_k(LaunchOpt(pdl_after_band(sc), sc.prio), k_leaf_up,
             blocks_for(leaf_threads, 288), 288, 0, st, x,
             (const double *)p->T, p->w, g);
    CK(cudaGetLastError());
  }
  if (!band(1)) return 0;
  const TreePlan tp = tree_plan(p->L, count, p->tree_l0);
  {
    PhaseScope ps(p, L2C_PHASE_TREE_UP, tree_launches(tp, p->L));
    CK(sweep_up(p->w, g, tp, st, LaunchOpt(sc.pdl & 1, sc.prio), p->nodal));
  }
  if (!band(2)) return 0;
  {
    PhaseScope ps(p, L2C_PHASE_FAR, 1);
    const long long n = g.count * (long long)p->Nb * M;  // both parities per thread
    launch_k(LaunchOpt(sc.pdl & 1, sc.prio), k_far, blocks_for(n, 256), 256,
             0, st, (const double *)p->A[dir],
             (const double *)p->w, p->c, g, (long long)p->Nb);
    CK(cudaGetLastError());
  }
  if (!band(3)) return 0;
  {
    PhaseScope ps(p, L2C_PHASE_TREE_DOWN, tree_launches(tp, p->L));
    CK(sweep_down(p->c, g, tp, st, LaunchOpt(sc.pdl & 1, sc.prio), p->nodal));
  }
  if (ov) CK(cudaStreamWaitEvent(st, p->ev_join, 0));
  {
    PhaseScope ps(p, L2C_PHASE_LEAF_DOWN, 1);
    launch_k((sc.pdl & 1) && !ov, k_leaf_down, blocks_for(total, 256), 256, 0, st,
             (const double *)p->c,
             (const double *)p->T, (const double *)p->y, out, g, c2l);
    CK(cudaGetLastError());
  }
  return 1;
}

// Launch choices -> the plan's fields.
void cfg_apply(l2c_gpu_plan *p, const TuneCfg &c) {
  p->overlap = c.overlap;
  p->pdl = c.pdl;
  p->chain_prio_mode = c.prio;
  p->near_threads = c.nthreads;
  p->near_vb = c.nvb;
  p->near_pair = c.npair;
  p->near_ctas = (unsigned)c.nctas;
  p->oz_nbuf = c.nbuf;
  p->band_fork = c.fork;
  p->mz_top_lvl = c.mtop;
  p->mz_top_g = c.mtopg > 0 ? c.mtopg : p->mz_top_g_base;
  p->tree_l0 = c.tl0;
  p->band_bseg = c.bseg;
  p->far_split = c.fsplit;
  p->band_thin = c.bthin;
  p->far_tc = c.fartc;
  p->oz_ld_ctas = p->oz_ld_ctas_nb[c.nbuf == 2 ? 2 : 1];
  p->cfg_cur = c;
}

// Whether a call's band reads the weight table (TuneCfg::wtab).
bool wants_table(const l2c_gpu_plan *p, const TuneCfg &c, size_t count) {
  if (p->L == 0 || c.wtab == 0) return false;
  if (c.wtab == 1 || p->precompute) return true;
  return count > 1 && near_table_size(p->N, p->s) <= count * p->N;
}

// The band weights of one direction, built on first use (outside any capture).
bool ensure_near_table(l2c_gpu_plan *p, size_t dir) {
  if (p->Wnear[dir]) return true;
  const size_t nw = near_table_size(p->N, p->s);
  if (cudaMalloc(&p->Wnear[dir], nw * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    p->Wnear[dir] = nullptr;
    set_err("cudaMalloc of the band weight table failed");
    return false;
  }
  Geo g = make_geo(p, 1, p->N, 1);
  k_near_weights<<<blocks_for((long long)p->N, 256), 256, 0, p->stream>>>(p->Wnear[dir], p->a,
                                                                          p->an, p->dn, g,
                                                                          (int)dir);
  return cudaGetLastError() == cudaSuccess;
}

// The dense band weights of one direction for k_band_tile, built on first use
// (outside any capture).  The same products as the compact table, so the band
// gives the same bits with either table or none.
bool ensure_band_tile_table(l2c_gpu_plan *p, size_t dir) {
  if (p->Wtile[dir]) return true;
  const size_t nw = band_tile_table_size(p->N, p->s);
  if (cudaMalloc(&p->Wtile[dir], nw * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    p->Wtile[dir] = nullptr;
    set_err("cudaMalloc of the tiled band weight table failed");
    return false;
  }
  Geo g = make_geo(p, 1, p->N, 1);
  k_band_tile_weights<<<blocks_for((long long)nw, 256), 256, 0, p->stream>>>(
      p->Wtile[dir], p->a, p->an, p->dn, g, (int)dir);
  return cudaGetLastError() == cudaSuccess;
}

size_t shape_dist(size_t count, size_t dist) { return count > 1 ? dist : 0; }

const TunedShape *tuned_for(const l2c_gpu_plan *p, size_t dir, size_t count, size_t dist,
                            size_t stride) {
  const size_t d = shape_dist(count, dist);
  for (auto it = p->tuned.rbegin(); it != p->tuned.rend(); ++it)
    if (it->dir == dir && it->count == count && it->dist == d && it->stride == stride) return &*it;
  return nullptr;
}

// Device-pointer execution of one batch: replay a captured graph of the launch
// sequence when one exists for this call shape, else capture one (or launch
// directly while per-phase profiling is on).  The launch choices are the
// tuned ones of the shape when it has been tuned, else the plan's own.
size_t run_device(l2c_gpu_plan *p, const double *in, double *out, size_t dir, size_t count,
                  size_t dist, size_t stride, bool near_only, bool input_ready,
                  bool in_host = false) {
  if (count == 0 || p->N == 0) return 1;
  {
    const TunedShape *ts = p->forced ? nullptr : tuned_for(p, dir, count, dist, stride);
    const TuneCfg &c = p->forced ? *p->forced : ts ? ts->cfg : p->base;
    cfg_apply(p, c);
    p->use_w = wants_table(p, c, count);
    if (p->use_w && (use_band_tile(p, count) || use_near_rows(p, count))) {
      if (!ensure_band_tile_table(p, dir)) return 0;
    } else if (p->use_w && !ensure_near_table(p, dir)) {
      return 0;
    }
  }
  if (!ensure_scratch(p, count)) return 0;
  if (p->mixed && p->L > 0 && count >= 4 && !ensure_mixed_far(p, dir)) return 0;
  if (p->mixed && p->L > 0 && count >= 4 && far_tc_on(p) && !ensure_mixed_far_tc(p, dir))
    return 0;
  if (use_mz_band(p, count) && !ensure_mz_band(p, dir)) return 0;
  const unsigned mode = (near_only ? 1u : 0u) | (input_ready ? 2u : 0u) | (in_host ? 4u : 0u);
  if (p->profiling || !p->use_graphs) {
    return launch_all(p, in, out, dir, count, dist, stride, near_only, input_ready, in_host);
  }
  p->use_clock++;
  for (auto &e : p->graphs) {
    if (e.dir == dir && e.count == count && e.dist == dist && e.stride == stride && e.in == in &&
        e.out == out && e.mode == mode && e.use_w == p->use_w && same_cfg(e.cfg, p->cfg_cur)) {
      e.last_use = p->use_clock;
      CK(cudaGraphLaunch(e.exec, p->stream));
      p->launches += e.launches;
      return 1;
    }
  }
  const size_t before = p->launches;
  CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
  const size_t ok =
      launch_all(p, in, out, dir, count, dist, stride, near_only, input_ready, in_host);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(p->stream, &graph);
  if (!ok || ec != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    if (!ok) return 0;
    set_err("stream capture failed: %s", cudaGetErrorString(ec));
    return 0;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei =
      cudaGraphInstantiate(&exec, graph, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) {
    set_err("cudaGraphInstantiate failed: %s", cudaGetErrorString(ei));
    return 0;
  }
  l2c_gpu_plan::GraphEntry e{dir,        count,    dist, stride, in,
                             out,        mode,     p->cfg_cur, p->use_w, exec,
                             p->launches - before, p->use_clock};
  if (p->graphs.size() >= 8) {
    auto oldest = std::min_element(p->graphs.begin(), p->graphs.end(),
                                   [](const l2c_gpu_plan::GraphEntry &a,
                                      const l2c_gpu_plan::GraphEntry &b) {
                                     return a.last_use < b.last_use;
                                   });
    cudaGraphExecDestroy(oldest->exec);
    p->graphs.erase(oldest);
  }
  p->graphs.push_back(e);
  CK(cudaGraphLaunch(exec, p->stream));
  return 1;
}

// ---------------------------------------------------------------------------
// Autotuner.  For one call shape (direction, count, dist, stride) it times the
// launch choices of TuneCfg -- none of which changes results -- on synthetic
// device data and keeps the fastest: coordinate descent from the plan's own
// choices, one choice at a time over its values, a change kept when it saves
// at least 1 %, until a pass keeps none (two passes at most).  Each timing is
// the captured graph of the call (captured and replayed twice first), the best
// of three runs of three calls, by CUDA events on the plan's stream (which the
// band's stream joins).  Tuned shapes are kept in the plan and, with
// L2C_AUTOTUNE_CACHE=path, appended to that file and read back by later plans
// of the same device, N, maxs and form.
// ---------------------------------------------------------------------------

// Uniform [-1, 1) from a counter (splitmix64's output function).
__global__ void k_tune_fill(double *v, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long z = (unsigned long long)i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  v[i] = (double)(z >> 11) * 0x1.0p-52 - 1.0;
}

// ms per call under c (< 0 on error).
// One configuration's time per call: after capture and two warm-up replays,
// the best of three runs of three calls.  Each timed call starts from an L2
// that another buffer has just filled (flush, flush_bytes; none if null), as a
// call does whose inputs and tables were not the last thing the GPU touched:
// with the tables warm in L2 the chain looked shorter than it is and the
// search favoured the wrong fork point for large single vectors.
double tune_time(l2c_gpu_plan *p, const double *in, double *out, size_t dir, size_t count,
                 size_t dist, size_t stride, const TuneCfg &c, cudaEvent_t e0, cudaEvent_t e1,
                 void *flush, size_t flush_bytes) {
  p->forced = &c;
  double best = -1.0;
  bool ok = true;
  for (int i = 0; i < 2 && ok; i++)
    ok = run_device(p, in, out, dir, count, dist, stride, false, false) != 0;
  for (int rep = 0; rep < 3 && ok; rep++) {
    double sum = 0.0;
    for (int i = 0; i < 3 && ok; i++) {
      if (flush)
        ok = cudaMemsetAsync(flush, (rep * 3 + i) & 0xff, flush_bytes, p->stream) == cudaSuccess;
      ok = ok && cudaEventRecord(e0, p->stream) == cudaSuccess;
      ok = ok && run_device(p, in, out, dir, count, dist, stride, false, false) != 0;
      float ms = 0.f;
      ok = ok && cudaEventRecord(e1, p->stream) == cudaSuccess &&
           cudaEventSynchronize(e1) == cudaSuccess &&
           cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      sum += ms;
    }
    if (ok && (best < 0.0 || sum / 3.0 < best)) best = sum / 3.0;
  }
  p->forced = nullptr;
  return ok ? best : -1.0;
}

// The plan's own choices for a shape, with the "by shape" ones resolved as
// sched_for and near_pair resolve them.
TuneCfg resolved_cfg(l2c_gpu_plan *p, size_t count) {
  cfg_apply(p, p->base);
  const Sched sc = sched_for(p, count);
  TuneCfg c = p->base;
  c.overlap = sc.ov ? 1 : 0;
  c.pdl = (int)sc.pdl;
  c.prio = p->chain_prio_mode >= 0
               ? p->chain_prio_mode
               : ((p->mixed || count == 1) && band_fork_for(p, count) == 0 ? 1 : 0);
  c.fork = band_fork_for(p, count);
  return c;
}

void cfg_text(const TuneCfg &c, char *buf, size_t len) {
  snprintf(buf, len, "overlap=%d band_fork=%d pdl=%d prio=%d near_threads=%d near_vb=%d "
           "near_pair=%d near_ctas=%d nbuf=%d near_table=%d mz_top=%d mz_top_g=%d tree_l0=%d "
           "band_bseg=%d far_split=%d band_thin=%d far_tc=%d", c.overlap, c.fork, c.pdl, c.prio,
           c.nthreads, c.nvb, c.npair, c.nctas, c.nbuf, c.wtab, c.mtop, c.mtopg, c.tl0, c.bseg,
           c.fsplit, c.bthin, c.fartc);
}

// Cache file: one line per tuned shape, fields separated by '|':
// l2c-tune-6|device|SMs|N|maxs|form|precompute|dir|count|dist|stride|
//   overlap|pdl|prio|nthreads|nvb|npair|nctas|nbuf|wtab|fork|mtop|mtopg|tl0|bseg|
//   fsplit|bthin|fartc|ms|ms_default
// (form 0 modal, 1 nodal, 2 mixed).  Later lines win.
constexpr int TUNE_FIELDS = 30;

struct TuneKey {
  char dev[256];
  int sms;
  int form, pre;
};

TuneKey tune_key(const l2c_gpu_plan *p) {
  TuneKey k{};
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, p->device) == cudaSuccess) {
    snprintf(k.dev, sizeof(k.dev), "%s", prop.name);
    k.sms = prop.multiProcessorCount;
  } else {
    cudaGetLastError();
    snprintf(k.dev, sizeof(k.dev), "unknown");
  }
  for (char *c = k.dev; *c; c++)
    if (*c == '|' || *c == '\n') *c = ' ';
  k.form = p->mixed ? 2 : p->nodal ? 1 : 0;
  k.pre = p->precompute ? 1 : 0;
  return k;
}

void cache_append(const l2c_gpu_plan *p, const TunedShape &t) {
  if (!p->tune_cache[0]) return;
  const TuneKey k = tune_key(p);
  FILE *f = std::fopen(p->tune_cache, "a");
  if (!f) return;  // an unwritable cache leaves the tuning in the plan only
  const TuneCfg &c = t.cfg;
  std::fprintf(f,
               "l2c-tune-6|%s|%d|%zu|%zu|%d|%d|%zu|%zu|%zu|%zu|%d|%d|%d|%d|%d|%d|%d|%d|%d|%d|"
               "%d|%d|%d|%d|%d|%d|%d|%.6f|%.6f\n",
               k.dev, k.sms, p->N, p->maxs, k.form, k.pre, t.dir, t.count, t.dist, t.stride,
               c.overlap, c.pdl, c.prio, c.nthreads, c.nvb, c.npair, c.nctas, c.nbuf, c.wtab,
               c.fork, c.mtop, c.mtopg, c.tl0, c.bseg, c.fsplit, c.bthin, c.fartc, t.ms,
               t.ms_default);
  std::fclose(f);
}

// Entries of the cache file for this plan (device, N, maxs, form, precompute);
// malformed or foreign lines are skipped.
void cache_load(l2c_gpu_plan *p) {
  if (!p->tune_cache[0]) return;
  FILE *f = std::fopen(p->tune_cache, "r");
  if (!f) return;
  const TuneKey k = tune_key(p);
  char line[2048];
  while (std::fgets(line, sizeof(line), f)) {
    char *fld[TUNE_FIELDS];
    int n = 0;
    char *q = line;
    fld[n++] = q;
    for (; *q && n < TUNE_FIELDS; q++)
      if (*q == '|') {
        *q = 0;
        fld[n++] = q + 1;
      }
    if (n != TUNE_FIELDS || std::strcmp(fld[0], "l2c-tune-6") != 0) continue;
    if (std::strcmp(fld[1], k.dev) != 0 || std::atoi(fld[2]) != k.sms) continue;
    auto u = [&](int i) { return (size_t)std::strtoull(fld[i], nullptr, 10); };
    auto iv = [&](int i) { return (int)std::strtol(fld[i], nullptr, 10); };
    if (u(3) != p->N || u(4) != p->maxs || iv(5) != k.form || iv(6) != k.pre) continue;
    TunedShape t{};
    t.dir = u(7);
    t.count = u(8);
    t.dist = u(9);
    t.stride = u(10);
    t.cfg.overlap = iv(11);
    t.cfg.pdl = iv(12);
    t.cfg.prio = iv(13);
    t.cfg.nthreads = iv(14);
    t.cfg.nvb = iv(15);
    t.cfg.npair = iv(16);
    t.cfg.nctas = iv(17);
    t.cfg.nbuf = iv(18);
    t.cfg.wtab = iv(19);
    t.cfg.fork = iv(20);
    t.cfg.mtop = iv(21);
    t.cfg.mtopg = iv(22);
    t.cfg.tl0 = iv(23);
    t.cfg.bseg = iv(24);
    t.cfg.fsplit = iv(25);
    t.cfg.bthin = iv(26);
    t.cfg.fartc = iv(27);
    t.ms = std::strtod(fld[28], nullptr);
    t.ms_default = std::strtod(fld[29], nullptr);
    t.from_cache = true;
    // only values the launches accept
    const TuneCfg &c = t.cfg;
    if (t.dir > 1 || t.count == 0 || t.stride == 0 || c.overlap < 0 || c.overlap > 1 ||
        c.pdl < 0 || c.pdl > 7 || c.prio < 0 || c.prio > 1 ||
        (c.nthreads != 128 && c.nthreads != 256) || c.nvb < 1 || c.nvb > 8 || c.npair < -1 ||
        c.npair > 1 || c.nctas < 0 || c.nbuf < 1 || c.nbuf > 2 || c.wtab < -1 || c.wtab > 1 ||
        c.fork < 0 || c.fork > 3 || c.mtop < -2 || c.mtop > 5 || c.mtopg < 0 || c.mtopg > 7 ||
        c.tl0 < -1 || c.tl0 > 14 || c.bseg < 0 || c.bseg > 31 || c.fsplit < -1 ||
        c.fsplit > FAR_SPLIT_MAX || c.bthin < -1 || c.bthin > 1 || c.fartc < -1 || c.fartc > 1)
      continue;
    p->tuned.push_back(t);
  }
  std::fclose(f);
}

void ensure_tune_cache(l2c_gpu_plan *p) {
  if (p->tune_cache_loaded) return;
  p->tune_cache_loaded = true;
  cache_load(p);
}

// Tunes one call shape; returns the tuned ms per call (0 on error).
double tune_shape(l2c_gpu_plan *p, size_t dir, size_t count, size_t dist, size_t stride) {
  if (stride == 0) stride = 1;
  if (count > 1 && dist == 0) {
    set_err("dist must be positive for count > 1");
    return 0.0;
  }
  const size_t span = (count - 1) * dist + (p->N - 1) * stride + 1;
  double *din = nullptr, *dout = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double result = 0.0;
  int sms = 152, l2 = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
  cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, p->device);
  // a buffer twice the L2 to write before each timed call (none if it cannot
  // be had: the timings are then taken with warm caches)
  void *flush = nullptr;
  const size_t flush_bytes = std::max<size_t>(2 * (size_t)l2, (size_t)64 << 20);
  if (cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
    cudaGetLastError();
    flush = nullptr;
  }
  if (cudaMalloc(&din, span * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dout, span * sizeof(double)) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    set_err("autotuner: device allocation failed");
  } else {
    k_tune_fill<<<blocks_for((long long)span, 256), 256, 0, p->stream>>>(din, (long long)span);
    cudaMemsetAsync(dout, 0, span * sizeof(double), p->stream);
    TuneCfg cur = resolved_cfg(p, count);
    const TuneCfg dflt = cur;
    // a first timing brings the GPU's clocks up (the first shape tuned after
    // an idle spell read ~15 % slow) and is dropped
    tune_time(p, din, dout, dir, count, dist, stride, cur, e0, e1, flush,
              flush_bytes);
    double t_default = tune_time(p, din, dout, dir, count, dist, stride, cur, e0, e1, flush,
                                 flush_bytes);
    double best = t_default;
    if (best > 0.0 && p->L > 0) {
      struct Knob {
        int TuneCfg::*f;
        std::vector<int> vals;
      };
      const bool tile = use_band_tile(p, count);
      std::vector<Knob> knobs = {{&TuneCfg::overlap, {0, 1}},
                                 {&TuneCfg::fork, {0, 1, 2, 3}},
                                 {&TuneCfg::pdl, {0, 1, 7}},
                                 {&TuneCfg::prio, {0, 1}}};
      if (tile) {
        // k_band_tile's grid: 0 = two CTAs per SM, one, or three
        knobs.push_back({&TuneCfg::nctas, {0, sms, 3 * sms}});
      } else {
        knobs.push_back({&TuneCfg::nthreads, {128, 256}});
        knobs.push_back({&TuneCfg::nctas, {0, 3 * sms, 6 * sms}});
        if (count > 1) knobs.push_back({&TuneCfg::nvb, {1, 2, 4, 8}});
      }
      // the weight table: when the plan has one, or a batch's would be small
      if (p->precompute || (count > 1 && near_table_size(p->N, p->s) <= count * p->N))
        knobs.push_back({&TuneCfg::wtab, {0, 1}});
      if (p->mixed) knobs.push_back({&TuneCfg::nbuf, {1, 2}});
      // the per-level structure: the mixed form's top launch (its coarsest
      // level and trees per CTA), the plain form's subtree roots, the tiled
      // band's blocks per work unit
      if (p->mixed && p->L >= 4) {
        knobs.push_back({&TuneCfg::mtop, {-2, -1, 3, 5}});
        knobs.push_back({&TuneCfg::mtopg, {0, 1, 4}});
      }
      if (!p->mixed && p->L >= 4) {
        const int l0 = tree_plan(p->L, count).l0;
        std::vector<int> v = {-1};
        for (int d = -2; d <= 2; d++)
          if (d != 0 && l0 + d >= 0 && l0 + d <= (int)p->L - 2) v.push_back(l0 + d);
        knobs.push_back({&TuneCfg::tl0, v});
      }
      if (tile) knobs.push_back({&TuneCfg::bseg, {0, 1, 2, 4}});
      if (tile && p->s == 16) knobs.push_back({&TuneCfg::bthin, {0, 1}});
      if (p->mixed && count >= 4 && p->L >= 3) knobs.push_back({&TuneCfg::fsplit, {0, 1, 2, 3}});
      // the tensor-memory far field, where its fragment copy (27 KB per block
      // and direction) stays under 1 GB
      if (p->mixed && count >= 4 && p->L >= 2 &&
          p->Nb * (size_t)FTC_B_WORDS * sizeof(unsigned) <= ((size_t)1 << 30))
        knobs.push_back({&TuneCfg::fartc, {0, 1}});
      for (int pass = 0; pass < 2 && best > 0.0; pass++) {
        bool kept = false;
        for (const Knob &kb : knobs)
          for (int v : kb.vals) {
            if (cur.*(kb.f) == v) continue;
            TuneCfg c = cur;
            c.*(kb.f) = v;
            const double t = tune_time(p, din, dout, dir, count, dist, stride, c, e0, e1, flush,
                                       flush_bytes);
            if (t < 0.0) {
              best = -1.0;
              break;
            }
            if (t < 0.99 * best) {
              best = t;
              cur = c;
              kept = true;
            }
          }
        if (!kept) break;
      }
      // confirmation: the plan's choices and the search's, timed again in
      // turn; the search's stay only if they still save 1 %
      if (best > 0.0 && !same_cfg(cur, dflt)) {
        double td = -1.0, tc = -1.0;
        for (int r = 0; r < 2 && best > 0.0; r++) {
          const double a = tune_time(p, din, dout, dir, count, dist, stride, dflt, e0, e1, flush,
                                     flush_bytes);
          const double b = tune_time(p, din, dout, dir, count, dist, stride, cur, e0, e1, flush,
                                     flush_bytes);
          if (a < 0.0 || b < 0.0) {
            best = -1.0;
          } else {
            td = td < 0.0 ? a : std::min(td, a);
            tc = tc < 0.0 ? b : std::min(tc, b);
          }
        }
        if (best > 0.0) {
          t_default = td;
          if (tc < 0.99 * td) {
            best = tc;
          } else {
            cur = dflt;
            best = td;
          }
        }
      }
    }
    if (best > 0.0) {
      TunedShape t{dir, count, shape_dist(count, dist), stride, cur, best, t_default, false};
      p->tuned.erase(std::remove_if(p->tuned.begin(), p->tuned.end(),
                                    [&](const TunedShape &o) {
                                      return o.dir == t.dir && o.count == t.count &&
                                             o.dist == t.dist && o.stride == t.stride;
                                    }),
                     p->tuned.end());
      p->tuned.push_back(t);
      cache_append(p, t);
      result = best;
    } else if (!g_err[0]) {
      set_err("autotuner: a timed call failed");
    }
  }
  // graphs captured on the tuning buffers go with them
  cudaStreamSynchronize(p->stream);
  cudaStreamSynchronize(p->stream2);
  cudaStreamSynchronize(p->stream3);
  for (auto it = p->graphs.begin(); it != p->graphs.end();) {
    if (it->in == din || it->out == dout) {
      cudaGraphExecDestroy(it->exec);
      it = p->graphs.erase(it);
    } else {
      ++it;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (din) cudaFree(din);
  if (dout) cudaFree(dout);
  if (flush) cudaFree(flush);
  return result;
}

}  // namespace

extern "C" {

size_t l2c_geometry(size_t N, size_t maxs, size_t *s_out, size_t *Nn_out) {
  // N = 0 or maxs = 0: no levels (and no log of zero or division by it)
  const int L = (N == 0 || maxs == 0) ? 0 : (int)std::ceil(std::log2((double)N / (double)maxs)) - 2;
  if (L < 1) {
    if (s_out) *s_out = 0;
    if (Nn_out) *Nn_out = N;
    return 0;
  }
  const size_t s = (size_t)std::ceil((double)N / std::pow(2.0, L + 2));
  if (s_out) *s_out = s;
  if (Nn_out) *Nn_out = s * ((size_t)1 << (L + 2));
  return (size_t)L;
}

l2c_gpu_plan *l2c_gpu_plan_create(size_t N, size_t maxs, size_t directions, unsigned flags) {
  g_err[0] = 0;
  if (N == 0) {
    set_err("N must be positive");
    return nullptr;
  }
  if (directions > 2) {
    set_err("direction must be 0 (L2C), 1 (C2L) or 2 (both)");
    return nullptr;
  }
  l2c_gpu_plan *p = new (std::nothrow) l2c_gpu_plan();
  if (!p) {
    set_err("out of host memory");
    return nullptr;
  }
  auto fail = [&]() -> l2c_gpu_plan * {
    l2c_gpu_plan_destroy(p);
    return nullptr;
  };
#define PCK(call)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return fail();                                                                       \
    }                                                                                      \
  } while (0)
  p->N = N;
  p->maxs = maxs;
  p->dirs = directions;
  PCK(cudaGetDevice(&p->device));
  PCK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  PCK(cudaStreamCreateWithFlags(&p->stream2, cudaStreamNonBlocking));
  PCK(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
  PCK(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
  PCK(cudaStreamCreateWithFlags(&p->stream3, cudaStreamNonBlocking));
  for (int k = 0; k < FAR_SPLIT_MAX; k++) {
    PCK(cudaEventCreateWithFlags(&p->ev_ff[k], cudaEventDisableTiming));
    PCK(cudaEventCreateWithFlags(&p->ev_fj[k], cudaEventDisableTiming));
  }
  if (const char *env = std::getenv("L2C_NO_GRAPHS")) p->use_graphs = env[0] == '0';
  if (const char *env = std::getenv("L2C_OVERLAP")) p->overlap = env[0] == '1' ? 1 : 0;
  if (const char *env = std::getenv("L2C_NEAR_CTAS")) p->near_ctas = (unsigned)std::atoi(env);
  if (const char *env = std::getenv("L2C_NEAR_VB")) p->near_vb = std::max(1, std::atoi(env));
  if (const char *env = std::getenv("L2C_NEAR_THREADS"))
    p->near_threads = std::atoi(env) == 128 ? 128 : 256;
  if (const char *env = std::getenv("L2C_NEAR_PAIR")) p->near_pair = env[0] == '1' ? 1 : 0;
  if (const char *env = std::getenv("L2C_BAND_TILE")) p->band_tile = env[0] == '0' ? 0 : -1;
  if (const char *env = std::getenv("L2C_MZ_TOP")) p->mz_top = env[0] != '0';
  if (const char *env = std::getenv("L2C_NEAR_ROWS")) p->near_rows = env[0] == '0' ? 0 : 1;
  if (const char *env = std::getenv("L2C_MZ_TOP_G")) p->mz_top_g = std::max(1, std::atoi(env));
  p->mz_top_g_base = p->mz_top_g;
  PCK(cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device));
  if (const char *env = std::getenv("L2C_PDL")) p->pdl = std::max(0, std::atoi(env));
  if (const char *env = std::getenv("L2C_CHAIN_PRIO")) p->chain_prio_mode = env[0] == '1' ? 1 : 0;
  if (const char *env = std::getenv("L2C_MZ_NBUF")) p->oz_nbuf = env[0] == '1' ? 1 : 2;
  if (const char *env = std::getenv("L2C_ZERO_COPY")) p->zero_copy = env[0] != '0';
  if (const char *env = std::getenv("L2C_AUTOTUNE")) p->autotune = env[0] == '1';
  if (const char *env = std::getenv("L2C_AUTOTUNE_CACHE"))
    snprintf(p->tune_cache, sizeof(p->tune_cache), "%s", env);
  p->base = TuneCfg{p->overlap,    p->pdl,       p->chain_prio_mode, p->near_threads,
                    p->near_vb,    p->near_pair, (int)p->near_ctas,  p->oz_nbuf};
  if (const char *env = std::getenv("L2C_NEAR_TABLE")) p->base.wtab = env[0] == '1' ? 1 : 0;
  if (const char *env = std::getenv("L2C_BAND_FORK"))
    p->base.fork = std::min(3, std::max(0, std::atoi(env)));
  // the per-level structure (TuneCfg::mtop, mtopg, tl0, bseg)
  if (const char *env = std::getenv("L2C_MZ_TOP_LVL"))
    p->base.mtop = std::min(5, std::max(-2, std::atoi(env)));
  if (const char *env = std::getenv("L2C_TREE_L0"))
    p->base.tl0 = std::min(14, std::max(-1, std::atoi(env)));
  if (const char *env = std::getenv("L2C_BAND_BSEG"))
    p->base.bseg = std::min(31, std::max(0, std::atoi(env)));
  if (const char *env = std::getenv("L2C_FAR_SPLIT"))
    p->base.fsplit = std::min(FAR_SPLIT_MAX, std::max(-1, std::atoi(env)));
  if (const char *env = std::getenv("L2C_BAND_THIN")) p->base.bthin = env[0] == '1' ? 1 : 0;
  if (const char *env = std::getenv("L2C_FAR_TC")) p->base.fartc = env[0] == '1' ? 1 : 0;
  if (const char *env = std::getenv("L2C_MZ_BAND")) p->mz_band_on = env[0] != '0';
  if (const char *env = std::getenv("L2C_MZ_BAND_TPW"))
    p->mz_band_tpw = std::min(16, std::max(1, std::atoi(env)));
  if (const char *env = std::getenv("L2C_FAR_COLS")) {
    const int v = std::atoi(env);
    p->far_cols = v == OZ_FAR_COLS / 2 || v == OZ_FAR_COLS ? v : 0;
  }
  p->precompute = (flags & L2C_PLAN_PRECOMPUTE_NEAR) != 0;
  if (flags & L2C_PLAN_DIRECT_ONLY) {
    p->L = 0;
    p->Nn = N;
  } else {
    p->L = l2c_geometry(N, maxs, &p->s, &p->Nn);
  }
  cudaStream_t st = p->stream;
  const bool need_c2l = directions == 1 || directions == 2;
  PCK(cudaMalloc(&p->a, N * sizeof(double)));
  k_lambda_table<<<blocks_for((long long)(N + 7) / 8, 128), 128, 0, st>>>(p->a, N);
  PCK(cudaGetLastError());
  if (need_c2l) {
    PCK(cudaMalloc(&p->an, N * sizeof(double)));
    PCK(cudaMalloc(&p->dn, ((N + 1) / 2 + 1) * sizeof(double)));
    k_c2l_tables<<<blocks_for((long long)N, 256), 256, 0, st>>>(p->a, p->an, p->dn, N);
    PCK(cudaGetLastError());
  }
  if (p->L > 0) {
    const size_t L = p->L, s = p->s;
    p->h = 2 * s;
    p->nL = N / p->h;
    p->Nb = ((size_t)2 << L) - (L + 2);
    p->slots = 2 * p->Nb;
    p->K = slots_at(L - 1);
    // host-side constants: Chebyshev points and DCT cosines (libm, as the reference)
    double xj[M], cs[MM];
    for (int i = 0; i < M; i++) xj[i] = std::cos((i + 0.5) * M_PI / M);
    for (int k = 0; k < M; k++)
      for (int n = 0; n < M; n++) cs[k * M + n] = std::cos(M_PI * k * (n + 0.5) / M);
    PCK(cudaMemcpyToSymbolAsync(c_xj, xj, sizeof(xj), 0, cudaMemcpyHostToDevice, st));
    PCK(cudaMemcpyToSymbolAsync(c_dct, cs, sizeof(cs), 0, cudaMemcpyHostToDevice, st));
    p->nodal = (flags & L2C_PLAN_NODAL) != 0;
    if (p->nodal && (flags & L2C_PLAN_MIXED)) {
      set_err("the mixed form is implemented for the modal form only (lagrange = 0)");
      return fail();
    }
    std::vector<double> T(2 * s * M);
    if (p->nodal) {
      // barycentric Lagrange weights from the Chebyshev points to -1 + i/s,
      // rows normalised by their sums (leg2cheb.c:997-1031), and the child
      // interpolation matrices B0 | B1 (leg2cheb.c:1076-1100)
      double wj[M];
      for (int j = 0; j < M; j++) wj[j] = ((j % 2 == 0) ? 1 : -1) * std::sin((j + 0.5) * M_PI / M);
      for (size_t i = 0; i < s; i++) {
        const double xe = -1 + (double)(2 * i) / (double)s, xo = -1 + (double)(2 * i + 1) / (double)s;
        double sume = 0.0, sumo = 0.0;
        for (int j = 0; j < M; j++) {
          const double se = wj[j] / (xe - xj[j]), so = wj[j] / (xo - xj[j]);
          T[i * M + j] = se;
          T[(s + i) * M + j] = so;
          sume += se;
          sumo += so;
        }
        for (int j = 0; j < M; j++) {
          T[i * M + j] /= sume;
          T[(s + i) * M + j] /= sumo;
        }
      }
      for (int i = 0; i < M; i++) {
        const double x0 = (xj[i] - 1) / 2, x1 = (xj[i] + 1) / 2;
        double sum0 = 0.0, sum1 = 0.0;
        for (int j = 0; j < M; j++) {
          const double s0 = wj[j] / (x0 - xj[j]), s1 = wj[j] / (x1 - xj[j]);
          p->lagB[i * M + j] = s0;
          p->lagB[MM + i * M + j] = s1;
          sum0 += s0;
          sum1 += s1;
        }
        for (int j = 0; j < M; j++) {
          p->lagB[i * M + j] /= sum0;
          p->lagB[MM + i * M + j] /= sum1;
        }
      }
      PCK(cudaMemcpyToSymbolAsync(c_lag_B, p->lagB, sizeof(p->lagB), 0, cudaMemcpyHostToDevice, st));
    }
    // modal: Vandermonde T_j(-1 + i/s), i < 2s, rows split even | odd (leg2cheb.c:621-648)
    for (size_t i = 0; i < 2 * s && !p->nodal; i++) {
      double row[M];
      const double xv = -1 + (double)i / (double)s;
      const double x2 = 2 * xv;
      row[0] = 1;
      row[1] = xv;
      for (int j = 2; j < M; j++) row[j] = row[j - 1] * x2 - row[j - 2];
      const size_t r = (i % 2 == 0) ? i / 2 : s + i / 2;
      std::memcpy(&T[r * M], row, sizeof(row));
    }
    PCK(cudaMalloc(&p->T, T.size() * sizeof(double)));
    PCK(cudaMemcpyAsync(p->T, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    double *f0 = nullptr;
    PCK(cudaMalloc(&f0, 2 * L * MM * sizeof(double)));
    k_assemble_f0<<<(unsigned)(2 * L), MM, 0, st>>>(f0, L, s);
    cudaError_t e = cudaGetLastError();
    for (int d = 0; d < 2 && e == cudaSuccess; d++)
      if (directions == (size_t)d || directions == 2)
        e = cudaMalloc(&p->A[d], 3 * p->Nb * MM * sizeof(double));
    if (e == cudaSuccess) {
      // one CTA per (block, r); the grid is at most 3 (2^(L+1)) CTAs
      k_assemble_A<<<(unsigned)(3 * p->Nb), MM, 0, st>>>(f0, p->A[0], p->A[1], L, s,
                                                         p->nodal ? 1 : 0);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(f0);
    PCK(e);
    if (flags & L2C_PLAN_MIXED) {
      if (s > 64) {
        set_err("the mixed form supports leaf sizes s <= 64 (got s = %zu)", s);
        return fail();
      }
      p->mixed = true;
      const int KC = (int)((s + 7) / 8), npass = (int)((s + 15) / 16);
      p->oz_kc = KC;
      p->oz_npass = npass;
      // constant factors, sliced on the host into fragment words
      struct RowOf {  // P[n][k] = base[n * rs + k * cs]
        const double *base;
        long long rs, cs;
        __host__ __device__ double operator()(int k) const { return base[k * cs]; }
      };
      const double lower[NTRI] = L2C_BINOM_LOWER_INIT, upper[NTRI] = L2C_BINOM_UPPER_INIT;
      std::vector<double> Bu(M * 2 * M, 0.0), Bd(2 * M * M, 0.0);
      for (int m = 0; m < M; m++)
        for (int i = 0; i <= m; i++) {
          const double b = lower[m * (m + 1) / 2 + i];
          Bu[m * 2 * M + i] = b;
          Bu[m * 2 * M + M + i] = ((m + i) & 1) ? -b : b;
        }
      for (int i = 0, k = 0; i < M; i++)
        for (int j = i; j < M; j++, k++) {
          Bd[i * M + j] = upper[k];
          Bd[(M + i) * M + j] = ((j - i) & 1) ? -upper[k] : upper[k];
        }
      const int wlu = oz_words(OZ_NT, KC), wtu = oz_words(OZ_NT, 5), wtd = oz_words(OZ_NT, 3);
      std::vector<unsigned> lu(2 * wlu), tu(wtu), td(2 * wtd), ld(2 * npass * OZ_LD_WORDS);
      std::vector<int> lue(2 * OZ_ROWS), tue(OZ_ROWS), tde(2 * OZ_ROWS), lde(2 * npass * 16);
      std::vector<int> lum(2 * OZ_META), tum(OZ_META), tdm(2 * OZ_META);
      for (int sg = 0; sg < 2; sg++) {
        const double *Ts = T.data() + sg * s * M;  // T_sg(i, m) = Ts[i * M + m]
        for (int n = 0; n < OZ_ROWS; n++)          // leaf up: P[m][i] = T_sg(i, m)
          oz_pack_row(RowOf{Ts + (n < M ? n : 0), 0, M}, n < M, n, (int)s, OZ_NT, KC,
                      lu.data() + sg * wlu, lue.data() + sg * OZ_ROWS);
        for (int ps = 0; ps < npass; ps++)         // leaf down: P[i][m] = T_sg(i, m)
          for (int n = 0; n < 16; n++) {
            const size_t i = 16 * (size_t)ps + n;
            oz_pack_row(RowOf{Ts + (i < s ? i : 0) * M, 0, 1}, i < s, n, M, 2, 3,
                        ld.data() + (sg * npass + ps) * OZ_LD_WORDS,
                        lde.data() + (sg * npass + ps) * 16);
          }
      }
      for (int n = 0; n < OZ_ROWS; n++) {
        oz_pack_row(RowOf{Bu.data() + (n < M ? n : 0) * 2 * M, 0, 1}, n < M, n, 2 * M, OZ_NT, 5,
                    tu.data(), tue.data());
        for (int ch = 0; ch < 2; ch++)
          oz_pack_row(RowOf{Bd.data() + (ch * M + (n < M ? n : 0)) * M, 0, 1}, n < M, n, M, OZ_NT,
                      3, td.data() + ch * wtd, tde.data() + ch * OZ_ROWS);
      }
      for (int k = 0; k < 2; k++) {
        oz_meta(lue.data() + k * OZ_ROWS, lum.data() + k * OZ_META);
        oz_meta(tde.data() + k * OZ_ROWS, tdm.data() + k * OZ_META);
      }
      oz_meta(tue.data(), tum.data());
      // The transfer matrices are dyadic rationals with at most 17 significant
      // bits below each row's largest entry, so only their two leading digit
      // slices are non-zero: the tree kernels then form 11 of the 21 products.
      {
        const int qu = l2c_oz::used_slices(tu.data(), OZ_NT, 5);
        const int qd = std::max(l2c_oz::used_slices(td.data(), OZ_NT, 3),
                                l2c_oz::used_slices(td.data() + wtd, OZ_NT, 3));
        p->oz_tree_q = std::max(qu, qd) <= 2 ? 2 : l2c_oz::SLICES;
        // keep each down matrix's leading oz_tree_q slices, back to back
        const int nq = oz_tree_words(p->oz_tree_q, 3);
        if (nq < wtd) {
          std::copy(td.begin() + wtd, td.begin() + wtd + nq, td.begin() + nq);
          td.resize(2 * (size_t)nq);
        }
      }
      auto upload = [&](auto **dst, const auto &v) -> cudaError_t {
        const size_t bytes = v.size() * sizeof(v[0]);
        cudaError_t e = cudaMalloc(dst, bytes);
        if (e == cudaSuccess) e = cudaMemcpy(*dst, v.data(), bytes, cudaMemcpyHostToDevice);
        return e;
      };
      PCK(upload(&p->oz_lu, lu));
      PCK(upload(&p->oz_lum, lum));
      PCK(upload(&p->oz_tu, tu));
      PCK(upload(&p->oz_tum, tum));
      PCK(upload(&p->oz_td, td));
      PCK(upload(&p->oz_tdm, tdm));
      PCK(upload(&p->oz_ld, ld));
      PCK(upload(&p->oz_lde, lde));
      // kernels whose shared memory can pass the 48 KB default
      const cudaFuncAttribute smax = cudaFuncAttributeMaxDynamicSharedMemorySize;
      // (the attribute is per kernel, not per plan: the largest leaves, s = 64)
      PCK(cudaFuncSetAttribute(k_mz_leaf_down<1>, smax, (int)mz_leaf_down_smem(4, 1, 128)));
      PCK(cudaFuncSetAttribute(k_mz_leaf_down<2>, smax, (int)mz_leaf_down_smem(4, 2, 128)));
      // resident leaf-down CTAs per SM at this plan's leaf size (registers, shared
      // memory), for either tile-buffer depth
      PCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &p->oz_ld_ctas_nb[1], k_mz_leaf_down<1>, 32 * MXW,
          mz_leaf_down_smem(p->oz_npass, 1, (long long)p->h)));
      PCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &p->oz_ld_ctas_nb[2], k_mz_leaf_down<2>, 32 * MXW,
          mz_leaf_down_smem(p->oz_npass, 2, (long long)p->h)));
      for (int b = 1; b <= 2; b++) p->oz_ld_ctas_nb[b] = std::max(1, p->oz_ld_ctas_nb[b]);
      p->oz_ld_ctas = p->oz_ld_ctas_nb[p->oz_nbuf == 2 ? 2 : 1];
      PCK(cudaFuncSetAttribute(k_mz_tree_up<2, 1>, smax, (int)oz_tree_up_smem(2, 1)));
      PCK(cudaFuncSetAttribute(k_mz_tree_up<2, 2>, smax, (int)oz_tree_up_smem(2, 2)));
      PCK(cudaFuncSetAttribute(k_mz_tree_up<l2c_oz::SLICES, 1>, smax,
                               (int)oz_tree_up_smem(l2c_oz::SLICES, 1)));
      PCK(cudaFuncSetAttribute(k_mz_tree_up<l2c_oz::SLICES, 2>, smax,
                               (int)oz_tree_up_smem(l2c_oz::SLICES, 2)));
      PCK(cudaFuncSetAttribute(k_mz_tree_down<2, 1>, smax, (int)oz_tree_down_smem(2, 1)));
      PCK(cudaFuncSetAttribute(k_mz_tree_down<2, 2>, smax, (int)oz_tree_down_smem(2, 2)));
      PCK(cudaFuncSetAttribute(k_mz_tree_down<l2c_oz::SLICES, 1>, smax,
                               (int)oz_tree_down_smem(l2c_oz::SLICES, 1)));
      PCK(cudaFuncSetAttribute(k_mz_tree_down<l2c_oz::SLICES, 2>, smax,
                               (int)oz_tree_down_smem(l2c_oz::SLICES, 2)));
      PCK(cudaFuncSetAttribute(k_mz_tree_up<2, 1, true>, smax, (int)oz_tree_up_smem(2, 1)));
      PCK(cudaFuncSetAttribute(k_mz_tree_up<l2c_oz::SLICES, 1, true>, smax,
                               (int)oz_tree_up_smem(l2c_oz::SLICES, 1)));
      PCK(cudaFuncSetAttribute(k_mz_tree_down<2, 1, true>, smax, (int)oz_tree_down_smem(2, 1)));
      PCK(cudaFuncSetAttribute(k_mz_tree_down<l2c_oz::SLICES, 1, true>, smax,
                               (int)oz_tree_down_smem(l2c_oz::SLICES, 1)));
      PCK(cudaFuncSetAttribute(k_mz_far<1>, smax, (int)oz_far_smem(1)));
      PCK(cudaFuncSetAttribute(k_mz_far<2>, smax, (int)oz_far_smem(2)));
      PCK(cudaFuncSetAttribute(k_mz_far_tc, smax, (int)ftc_smem()));
      PCK(cudaFuncSetAttribute(k_mz_band, smax, (int)mz_band_smem()));
      PCK(cudaFuncSetAttribute(k_mz_band2, smax, (int)mz_band2_smem()));
#define L2C_MZ_ATTR(kc)                                                                     \
  PCK(cudaFuncSetAttribute(k_mz_leaf_up<kc, 1>, smax, (int)mz_leaf_up_smem(kc, 1)));        \
  PCK(cudaFuncSetAttribute(k_mz_leaf_up<kc, 2>, smax, (int)mz_leaf_up_smem(kc, 2)));
      L2C_MZ_ATTR(1) L2C_MZ_ATTR(2) L2C_MZ_ATTR(3) L2C_MZ_ATTR(4)
      L2C_MZ_ATTR(5) L2C_MZ_ATTR(6) L2C_MZ_ATTR(7) L2C_MZ_ATTR(8)
#undef L2C_MZ_ATTR
    }
    if (band_tile_ok((long long)s, (long long)p->nL, BT_MIN_COUNT)) {
      // the tiled band's three half-window slots can pass the 48 KB default
      const cudaFuncAttribute smax = cudaFuncAttributeMaxDynamicSharedMemorySize;
      for (bool thin : {false, true}) {
        const int bytes = (int)band_tile_smem((long long)s, thin);
        PCK(cudaFuncSetAttribute(band_tile_kernel<true>((long long)s, thin), smax, bytes));
        PCK(cudaFuncSetAttribute(band_tile_kernel<false>((long long)s, thin), smax, bytes));
      }
    }
    if (flags & L2C_PLAN_PRECOMPUTE_NEAR) {
      // the band weights now, in the dense layout single vectors and large
      // batches read (the per-output layout of other batches is built on its
      // first use); the same products either way
      const size_t nw = band_tile_table_size(N, s);
      Geo g = make_geo(p, 1, N, 1);
      for (int d = 0; d < 2 && nw > 0; d++) {
        if (!(directions == (size_t)d || directions == 2)) continue;
        PCK(cudaMalloc(&p->Wtile[d], nw * sizeof(double)));
        k_band_tile_weights<<<blocks_for((long long)nw, 256), 256, 0, st>>>(p->Wtile[d], p->a,
                                                                            p->an, p->dn, g, d);
        PCK(cudaGetLastError());
      }
    }
  }
  PCK(cudaStreamSynchronize(st));
  for (size_t d = 0; d < 2; d++)
    if (directions == d || directions == 2) p->flops[d] = ref_flops(p, d);
  {
    int least = 0, greatest = 0;
    PCK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    p->prio_greatest = greatest;
  }
  return p;
#undef PCK
}

void l2c_gpu_plan_destroy(l2c_gpu_plan *p) {
  if (!p) return;
  DeviceGuard dg(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->stream2) cudaStreamSynchronize(p->stream2);
  if (p->stream3) cudaStreamSynchronize(p->stream3);
  collect_profile(p);
  for (cudaEvent_t e : p->ev_pool) cudaEventDestroy(e);
  drop_graphs(p);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->ev_join) cudaEventDestroy(p->ev_join);
  for (int k = 0; k < FAR_SPLIT_MAX; k++) {
    if (p->ev_ff[k]) cudaEventDestroy(p->ev_ff[k]);
    if (p->ev_fj[k]) cudaEventDestroy(p->ev_fj[k]);
  }
  if (p->stream2) cudaStreamDestroy(p->stream2);
  if (p->stream3) cudaStreamDestroy(p->stream3);
  double *bufs[] = {p->a, p->an, p->dn, p->A[0], p->A[1], p->T, p->x, p->y, p->w, p->c,
                    p->st_in, p->st_out, p->Wnear[0], p->Wnear[1], p->Wtile[0], p->Wtile[1]};
  for (double *b : bufs)
    if (b) cudaFree(b);
  void *obufs[] = {p->oz_lu,     p->oz_tu,     p->oz_td,      p->oz_ld,      p->oz_lum,
                   p->oz_tum,    p->oz_tdm,    p->oz_lde,     p->oz_far[0],  p->oz_far[1],
                   p->oz_farm[0], p->oz_farm[1], p->wE,        p->cE,         p->bad,
                   p->oz_far_tc[0], p->oz_far_tc[1], p->mz_band[0], p->mz_band[1],
                   p->mz_bande[0], p->mz_bande[1]};
  for (void *b : obufs)
    if (b) cudaFree(b);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
}

int l2c_gpu_plan_info(const l2c_gpu_plan *p, size_t *info) {
  if (!p || !info) return 0;
  info[0] = p->N;
  info[1] = p->L;
  info[2] = p->s;
  info[3] = p->Nn;
  info[4] = p->Nb;
  info[5] = M;
  info[6] = p->dirs;
  info[7] = p->maxs;
  return 1;
}

size_t l2c_gpu_flops(const l2c_gpu_plan *p, size_t dir) { return (p && dir < 2) ? p->flops[dir] : 0; }

void *l2c_gpu_plan_stream(l2c_gpu_plan *p) { return p ? (void *)p->stream : nullptr; }

int l2c_gpu_synchronize(l2c_gpu_plan *p) {
  if (!p) return 1;
  DeviceGuard dg(p->device);
  cudaError_t e = cudaStreamSynchronize(p->stream);
  if (e != cudaSuccess) {
    set_err("cudaStreamSynchronize failed: %s", cudaGetErrorString(e));
    return 1;
  }
  return 0;
}

size_t l2c_gpu_execute(l2c_gpu_plan *p, const double *in, double *out, size_t dir, size_t count,
                       size_t dist, size_t stride, unsigned flags) {
  g_err[0] = 0;
  if (!p || !in || !out) {
    set_err("null plan or array");
    return 0;
  }
  if (dir > 1) {
    set_err("direction must be 0 (L2C) or 1 (C2L)");
    return 0;
  }
  if (!(p->dirs == dir || p->dirs == 2)) {
    set_err("direction %zu was not planned", dir);
    return 0;
  }
  if (stride == 0) stride = 1;
  if (count == 0) return 0;
  if (count > 1 && dist == 0) {
    set_err("dist must be positive for count > 1");
    return 0;
  }
  const bool near_only = (flags & L2C_EXEC_NEAR_ONLY) != 0;
  if (near_only && p->L == 0) {
    set_err("near-field only execution needs an FMM plan (L >= 1)");
    return 0;
  }
  std::lock_guard<std::mutex> lock(p->mu);
  DeviceGuard dg(p->device);
  // tuned launch choices: from the cache file, or tuned now (L2C_AUTOTUNE=1)
  ensure_tune_cache(p);
  if (p->autotune && p->L > 0 && !near_only && !p->profiling &&
      !tuned_for(p, dir, count, dist, stride) && tune_shape(p, dir, count, dist, stride) <= 0.0)
    return 0;
  const size_t N = p->N;
  // span of caller memory the call touches (the direct path also zeroes [0, N))
  size_t span = (count - 1) * dist + (N - 1) * stride + 1;
  if (p->L == 0) span = std::max(span, (count - 1) * dist + N);
  // directL semantics: contiguous, premultiplied input
  const bool in_contig = near_only && dir == 1;
  const size_t in_span = in_contig ? (count - 1) * dist + N : span;
  bool in_dev = is_device_ptr(in), out_dev = is_device_ptr(out);
  // Page-locked host buffers of an FMM transform are used in place through
  // their device mapping: the gather kernel reads the input once over the
  // host link, the band reads and the leaf-down kernel writes the output --
  // no staging copies around the transform (N = 2^20 single vector, L2C + C2L
  // through host buffers: 1.44e9 -> 1.66e9 coef/s).
  bool in_host = false, out_host = false;
  if (p->zero_copy && p->L > 0 && !near_only) {
    if (!in_dev)
      if (const void *m = mapped_host_ptr(in)) {
        in = static_cast<const double *>(m);
        in_dev = in_host = true;
      }
    if (!out_dev)
      if (void *m = mapped_host_ptr(out)) {
        out = static_cast<double *>(m);
        out_dev = out_host = true;
      }
  }
  // host memory involved: the call returns once the results are there
  const bool host_side = in_host || out_host || !in_dev || !out_dev;
  if (!in_dev || !out_dev) {
    // host memory: stage the touched span (the layout is kept, so the kernels
    // see the same dist/stride)
    if ((!in_dev && in_span > p->cap_st_in) || (!out_dev && span > p->cap_st_out)) {
      CK(cudaStreamSynchronize(p->stream));
      drop_graphs(p);
    }
    if (!in_dev && !grow(&p->st_in, &p->cap_st_in, in_span)) return 0;
    if (!out_dev && !grow(&p->st_out, &p->cap_st_out, span)) return 0;
    if (!in_dev)
      CK(cudaMemcpyAsync(p->st_in, in, in_span * sizeof(double), cudaMemcpyHostToDevice, p->stream));
    if (!out_dev)
      CK(cudaMemcpyAsync(p->st_out, out, span * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  }
  const double *din = in_dev ? in : p->st_in;
  double *dout = out_dev ? out : p->st_out;
  if (!run_device(p, din, dout, dir, count, dist, stride, near_only, in_contig, in_host)) return 0;
  if (!out_dev)
    CK(cudaMemcpyAsync(out, dout, span * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  if (!(flags & L2C_EXEC_ASYNC) || host_side) CK(cudaStreamSynchronize(p->stream));
  size_t f = p->flops[dir];
  if (near_only) f = 1;  // callers of directM/directL get their own count
  return f * count;
}

size_t l2c_gpu_launch_count(const l2c_gpu_plan *p) { return p ? p->launches : 0; }

double l2c_gpu_autotune(l2c_gpu_plan *p, size_t dir, size_t count, size_t dist, size_t stride) {
  g_err[0] = 0;
  if (!p) {
    set_err("null plan");
    return 0.0;
  }
  if (dir > 1 || !(p->dirs == dir || p->dirs == 2)) {
    set_err("direction %zu was not planned", dir);
    return 0.0;
  }
  if (count == 0) {
    set_err("count must be positive");
    return 0.0;
  }
  std::lock_guard<std::mutex> lock(p->mu);
  DeviceGuard dg(p->device);
  ensure_tune_cache(p);
  return tune_shape(p, dir, count, dist, stride == 0 ? 1 : stride);
}

int l2c_gpu_tuned_config(l2c_gpu_plan *p, size_t dir, size_t count, size_t dist, size_t stride,
                         char *buf, size_t len, double *ms) {
  if (!p) return -1;
  std::lock_guard<std::mutex> lock(p->mu);
  ensure_tune_cache(p);
  const TunedShape *t = tuned_for(p, dir, count, dist, stride == 0 ? 1 : stride);
  const TuneCfg c = t ? t->cfg : resolved_cfg(p, count);
  if (buf && len) cfg_text(c, buf, len);
  if (ms) {
    ms[0] = t ? t->ms : 0.0;
    ms[1] = t ? t->ms_default : 0.0;
  }
  return t ? (t->from_cache ? 2 : 1) : 0;
}

int l2c_gpu_profile(l2c_gpu_plan *p, int enable) {
  if (!p) return 1;
  std::lock_guard<std::mutex> lock(p->mu);
  DeviceGuard dg(p->device);
  cudaStreamSynchronize(p->stream);
  collect_profile(p);
  for (int i = 0; i < L2C_NPHASES; i++) {
    p->phase_ms[i] = 0.0;
    p->phase_launches[i] = 0;
  }
  p->profiling = enable != 0;
  return 0;
}

int l2c_gpu_profile_read(l2c_gpu_plan *p, double *ms, size_t *launches) {
  if (!p) return 0;
  std::lock_guard<std::mutex> lock(p->mu);
  DeviceGuard dg(p->device);
  collect_profile(p);
  for (int i = 0; i < L2C_NPHASES; i++) {
    if (ms) ms[i] = p->phase_ms[i];
    if (launches) launches[i] = p->phase_launches[i];
  }
  return L2C_NPHASES;
}

size_t l2c_gpu_plan_copy(const l2c_gpu_plan *p, int which, double *dst, size_t n_max) {
  if (!p || !dst) return 0;
  const double *src = nullptr;
  size_t n = 0;
  switch (which) {
    case 0:
    case 1:
      src = p->A[which];
      n = 3 * p->Nb * MM;
      break;
    case 2:
      src = p->a;
      n = p->N;
      break;
    case 3:
      src = p->an;
      n = p->N;
      break;
    case 4:
      src = p->dn;
      n = (p->N + 1) / 2;
      break;
    case 5:
      src = p->T;
      n = 2 * p->s * M;
      break;
    case 6:  // nodal transfer matrices B0 | B1 (host copy)
      if (!p->nodal) return 0;
      n = std::min(n_max, (size_t)(2 * MM));
      std::memcpy(dst, p->lagB, n * sizeof(double));
      return n;
    default:
      return 0;
  }
  if (!src) return 0;
  n = std::min(n, n_max);
  DeviceGuard dg(p->device);
  if (cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_err("copy of plan data failed");
    return 0;
  }
  return n;
}

double l2c_lambda(double z) { return l2c_lambda_eval(z); }

double l2c_lambda_int(size_t z) {
  static const double table[256] = L2C_LAMBDA_INT_INIT;
  if (z > 255) return l2c_lambda_eval((double)z);
  return table[z];
}

const char *l2c_gpu_last_error(void) { return g_err; }

const char *l2c_gpu_version(void) { return "l2c-gb300 0.1 (sm_103a, fp64)"; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Execution without any device allocation.
//
// Some callers cannot allocate device memory at the moment they transform:
// applications that reserve the whole device up front for their own memory
// pool, long-running solvers that must not pay allocation latency or risk an
// allocation failure inside a time step, and hosts that hand a library only
// pre-sized buffers.  l2c_gpu_execute_noalloc serves them.  It runs the same
// kernels as l2c_gpu_execute on device pointers, but its working buffers
// (gathered input, near-field partial sums, the two coefficient trees) live in
// the fixed array below instead of the plan's grown-on-demand scratch.  It calls
// no cudaMalloc, cudaFree or other allocating routine.
//
// The array is a file-scope __device__ object: every GPU on which this library
// is loaded holds it (L2C_NOALLOC_SCRATCH_DOUBLES doubles, 4 MiB) until the
// process exits.  Host code may not take its name as a device address; the
// device address is looked up once per device with cudaGetSymbolAddress.
// ---------------------------------------------------------------------------
namespace {

static __device__ __align__(256) double g_noalloc_scratch[L2C_NOALLOC_SCRATCH_DOUBLES];

constexpr int kMaxDevices = 64;
double *g_noalloc_ptr[kMaxDevices] = {nullptr};
std::mutex g_noalloc_mu;
std::mutex g_noalloc_call_mu[kMaxDevices];  // one call at a time per device

// Doubles of scratch one transform needs: x and y (N each), w and c (2 parities
// x 2 N_b slots x 18 each).
size_t noalloc_need(const l2c_gpu_plan *p) { return 2 * p->N + 2 * (2 * p->slots * M); }

// Device address of the fixed scratch array on the current device (looked up on
// the first call per device).
double *noalloc_scratch_address(int dev) {
  if (dev < 0 || dev >= kMaxDevices) {
    set_err("device index %d out of range for the fixed scratch table", dev);
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      set_err("cudaGetSymbolAddress of the fixed scratch array failed: %s",
              cudaGetErrorString(e));
      return nullptr;
    }
    g_noalloc_ptr[dev] = static_cast<double *>(ptr);
  }
  return g_noalloc_ptr[dev];
}

}  // namespace


extern "C" size_t l2c_gpu_execute_noalloc(l2c_gpu_plan *p, const double *in, double *out,
                                          size_t dir, size_t stride) {
  g_err[0] = 0;
  if (!p || !in || !out) {
    set_err("null plan or array");
    return 0;
  }
  if (dir > 1 || !(p->dirs == dir || p->dirs == 2)) {
    set_err("direction %zu was not planned", dir);
    return 0;
  }
  if (p->L == 0) {
    set_err("l2c_gpu_execute_noalloc needs an FMM plan (L >= 1)");
    return 0;
  }
  if (stride == 0) stride = 1;
  const size_t need = noalloc_need(p);
  if (need > (size_t)L2C_NOALLOC_SCRATCH_DOUBLES) {
    set_err("plan needs %zu scratch doubles; the fixed array holds %zu (N = %zu is too large "
            "for l2c_gpu_execute_noalloc; use l2c_gpu_execute)",
            need, (size_t)L2C_NOALLOC_SCRATCH_DOUBLES, p->N);
    return 0;
  }
  if (!is_device_ptr(in) || !is_device_ptr(out)) {
    set_err("l2c_gpu_execute_noalloc takes device pointers only (staging host arrays would "
            "need device buffers)");
    return 0;
  }
  if (p->device < 0 || p->device >= kMaxDevices) {
    set_err("device index %d out of range", p->device);
    return 0;
  }
  // The fixed array is shared by every call in this process on this device: the
  // per-device lock, held until the work below has finished on the GPU, keeps
  // calls from overlapping (overlapping calls would race on the array).
  std::lock_guard<std::mutex> call_lock(g_noalloc_call_mu[p->device]);
  std::lock_guard<std::mutex> lock(p->mu);
  DeviceGuard dg(p->device);
  double *base = noalloc_scratch_address(p->device);
  if (!base) return 0;
  // every scratch element below is written before it is read within one call
  // (gather fills x, the band fills y, the leaf and upward kernels fill all of
  // w, the far-field kernel fills all of c), so nothing needs clearing
  double *x = base, *y = base + p->N;
  double *w = y + p->N, *c = w + 2 * p->slots * M;
  cudaStream_t st = p->stream;
  const int c2l = dir == 1;
  Geo g = make_geo(p, 1, p->N, stride);
  const long long total = g.N;
  k_gather<<<blocks_for(total, 256), 256, 0, st>>>(in, x, g, c2l);
  k_near<1><<<blocks_for(total, 256), 256, 0, st>>>(x, out, y, p->a, p->an, p->dn,
                                                    p->Wnear[dir], g, c2l, 0);
  k_leaf_up<<<blocks_for(g.K * 2 * M, 288), 288, 0, st>>>(x, p->T, w, g);
  for (long long l = (long long)p->L - 2; l >= 0; l--) {
    const long long np = (long long)slots_at((size_t)l);
    (p->nodal ? k_tree_up<true> : k_tree_up<false>)<<<blocks_for(2 * np, TREE_TILE), 32 * M, 0,
                                                      st>>>(
        w, g, 2 * (long long)blocks_before(l), 2 * (long long)blocks_before(l + 1), np);
  }
  k_far<<<blocks_for((long long)p->Nb * M, 256), 256, 0, st>>>(p->A[dir], w, c, g,
                                                               (long long)p->Nb);
  for (long long l = 0; l + 1 < (long long)p->L; l++) {
    const long long np = (long long)slots_at((size_t)l);
    (p->nodal ? k_tree_down<true> : k_tree_down<false>)<<<blocks_for(2 * np, TREE_TILE), 32 * M,
                                                          0, st>>>(
        c, g, 2 * (long long)blocks_before(l), 2 * (long long)blocks_before(l + 1), np);
  }
  k_leaf_down<<<blocks_for(total, 256), 256, 0, st>>>(c, p->T, y, out, g, c2l);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return p->flops[dir];
}

// ---------------------------------------------------------------------------
// Ragged batches: many vectors of different length N in one set of launches.
//
// For a fixed leaf size s the far-field blocks depend only on (s, depth below
// the top, block index): level l of an L-level plan is level l + (L' - L) of an
// L'-level plan with the same s, with the same leading blocks.  So one "donor"
// plan per distinct s, built with the largest level count among the vectors that
// use that s, supplies A, T and the Lambda tables (identical prefixes) for all of
// them.  Each phase is one launch over the concatenated work items of every
// vector; a thread finds its vector by binary search in the phase's prefix sums
// of item counts, so work is spread evenly over the SMs whatever the mix of N.
// ---------------------------------------------------------------------------
namespace {

struct RVec {
  Geo g;               // the vector's own geometry (count 1, stride 1)
  long long io;        // offset in the packed caller arrays and in x / y scratch
  long long wc;        // offset in the w / c scratch
  int donor;           // donor plan supplying tables
  int lshift;          // donor level = own level + lshift
  int direct;          // 1: O(N^2) direct method (L < 1)
};

struct RDonor {
  const double *a, *an, *dn, *T, *A[2];
  // dense band weights per direction (lists made with L2C_PLAN_PRECOMPUTE_NEAR):
  // block b of any vector with this leaf size is block b of the donor
  const double *Wt[2];
};

__device__ __forceinline__ int find_vec(const long long *__restrict__ pre, int nvec, long long idx) {
  int lo = 0, hi = nvec;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (pre[mid] <= idx) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void k_r_gather(const double *__restrict__ in, double *__restrict__ x,
                           const RVec *__restrict__ V, const long long *__restrict__ pre, int nvec,
                           int c2l) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= pre[nvec]) return;
  const int v = find_vec(pre, nvec, idx);
  const RVec &r = V[v];
  if (r.direct) return;
  gather_item(in + r.io, x + r.io, 1, c2l, idx - pre[v]);
}

// The band of every FMM vector with register windows (near_rows_item): items
// counted by pre (near_rows_items per vector, 0 for direct-method vectors).
// TAB: the band weights from the donors' dense tables (the same products, so
// the same bits as forming them here).
template <bool TAB>
__global__ void __launch_bounds__(256) k_r_near_rows(const double *__restrict__ x,
                                                     const double *out, double *__restrict__ y,
                                                     const RVec *__restrict__ V,
                                                     const RDonor *__restrict__ D,
                                                     const long long *__restrict__ pre, int nvec,
                                                     int c2l) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= pre[nvec]) return;
  const int v = find_vec(pre, nvec, idx);
  const RVec &r = V[v];
  if (r.direct) return;
  const RDonor &d = D[r.donor];
  near_rows_item<TAB>(x + r.io, out + r.io, y + r.io, d.a, d.an, d.dn, TAB ? d.Wt[c2l] : nullptr,
                      r.g, c2l, idx - pre[v]);
}

__global__ void __launch_bounds__(256) k_r_near(const double *__restrict__ x, const double *out,
                                                double *__restrict__ y,
                                                const RVec *__restrict__ V,
                                                const RDonor *__restrict__ D,
                                                const long long *__restrict__ pre, int nvec,
                                                int c2l) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= pre[nvec]) return;
  const int v = find_vec(pre, nvec, idx);
  const RVec &r = V[v];
  if (r.direct) return;
  const long long j = idx - pre[v];
  const RDonor &d = D[r.donor];
  double res[1];
  near_sums<1>(x + r.io + j, 0, d.a, d.an, d.dn, nullptr, r.g, c2l, j, res);
  y[r.io + j] = out[r.io + j] + res[0];
}

__global__ void __launch_bounds__(288) k_r_leaf_up(const double *__restrict__ x,
                                                   double *__restrict__ w,
                                                   const RVec *__restrict__ V,
                                                   const RDonor *__restrict__ D,
                                                   const long long *__restrict__ pre, int nvec) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= pre[nvec]) return;
  const int v = find_vec(pre, nvec, idx);
  const RVec &r = V[v];
  const long long rem0 = idx - pre[v];
  const long long node = rem0 / (2 * M);
  const long long rem = rem0 - node * 2 * M;
  leaf_up_item(x + r.io, D[r.donor].T, w + r.wc, r.g, node, (int)(rem / M), (int)(rem % M));
}

// depth d below the leaf level: vector parent level l = L - 1 - d; items are
// (vector, parity, parent slot), 2 S(l) per vector
__global__ void __launch_bounds__(32 * M) k_r_tree_up(double *w, const RVec *__restrict__ V,
                                                      const long long *__restrict__ pre, int nvec,
                                                      int d) {
  __shared__ double sB[NTRI];
  __shared__ double sx[TREE_TILE * TREE_PAD];
  __shared__ const double *child[TREE_TILE];
  __shared__ double *par[TREE_TILE];
  for (int t = threadIdx.x; t < NTRI; t += blockDim.x) sB[t] = c_binom_lower[t];
  if (threadIdx.x < TREE_TILE) {
    const long long idx = (long long)blockIdx.x * TREE_TILE + threadIdx.x;
    par[threadIdx.x] = nullptr;
    child[threadIdx.x] = w;
    if (idx < pre[nvec]) {
      const int v = find_vec(pre, nvec, idx);
      const RVec &r = V[v];
      const long long l = r.g.L - 1 - d;
      const long long np = (long long)slots_at((size_t)l);
      const long long q = idx - pre[v];
      const long long sg = q / np, jp = q - sg * np;
      double *ws = w + r.wc + sg * r.g.slots * M;
      child[threadIdx.x] = ws + (2 * (long long)blocks_before((size_t)l + 1) + 2 * jp + 2) * M;
      par[threadIdx.x] = ws + (2 * (long long)blocks_before((size_t)l) + jp) * M;
    }
  }
  __syncthreads();
  tree_up_tile(child, par, sB, sx);
}

__global__ void __launch_bounds__(256) k_r_far(const double *__restrict__ w,
                                               double *__restrict__ c,
                                               const RVec *__restrict__ V,
                                               const RDonor *__restrict__ D,
                                               const long long *__restrict__ pre, int nvec,
                                               int dir) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= pre[nvec]) return;
  const int v = find_vec(pre, nvec, idx);
  const RVec &r = V[v];
  const long long nb = r.g.slots / 2;
  const long long rem = idx - pre[v];
  const int sg = (int)(rem / (nb * M));
  const long long q = rem - sg * nb * M;
  const long long gb = q / M;
  const int m = (int)(q - gb * M);
  long long l = 0;
  while (l + 1 < r.g.L && (long long)blocks_before((size_t)l + 1) <= gb) l++;
  const long long gd = (long long)blocks_before((size_t)(l + r.lshift)) + gb -
                       (long long)blocks_before((size_t)l);
  const long long off = r.wc + sg * r.g.slots * M;
  far_item(D[r.donor].A[dir] + 3 * gd * MM, w + off, c + off, gb, m);
}

// level l (from the top) into level l + 1; items (vector, parity, parent slot)
__global__ void __launch_bounds__(32 * M) k_r_tree_down(double *c, const RVec *__restrict__ V,
                                                        const long long *__restrict__ pre,
                                                        int nvec, int l) {
  __shared__ double sB[NTRI];
  __shared__ double sx[TREE_TILE * TREE_PAD];
  __shared__ const double *par[TREE_TILE];
  __shared__ double *child[TREE_TILE];
  for (int t = threadIdx.x; t < NTRI; t += blockDim.x) sB[t] = c_binom_upper[t];
  if (threadIdx.x < TREE_TILE) {
    const long long idx = (long long)blockIdx.x * TREE_TILE + threadIdx.x;
    child[threadIdx.x] = nullptr;
    par[threadIdx.x] = c;
    if (idx < pre[nvec]) {
      const int v = find_vec(pre, nvec, idx);
      const RVec &r = V[v];
      const long long np = (long long)slots_at((size_t)l);
      const long long q = idx - pre[v];
      const long long sg = q / np, tp = q - sg * np;
      double *cs = c + r.wc + sg * r.g.slots * M;
      par[threadIdx.x] = cs + (2 * (long long)blocks_before((size_t)l) + tp) * M;
      child[threadIdx.x] = cs + (2 * (long long)blocks_before((size_t)l + 1) + 2 * tp) * M;
    }
  }
  __syncthreads();
  tree_down_tile(par, child, sB, sx);
}

__global__ void __launch_bounds__(256) k_r_leaf_down(const double *__restrict__ c,
                                                     const double *__restrict__ y, double *out,
                                                     const RVec *__restrict__ V,
                                                     const RDonor *__restrict__ D,
                                                     const long long *__restrict__ pre, int nvec,
                                                     int c2l) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= pre[nvec]) return;
  const int v = find_vec(pre, nvec, idx);
  const RVec &r = V[v];
  if (r.direct) return;
  leaf_down_item(c + r.wc, D[r.donor].T, y + r.io, out + r.io, r.g, c2l, idx - pre[v]);
}

__global__ void __launch_bounds__(256) k_r_direct(const double *in, double *out,
                                                  const RVec *__restrict__ V,
                                                  const RDonor *__restrict__ D,
                                                  const long long *__restrict__ pre, int nvec,
                                                  int c2l) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= pre[nvec]) return;
  const int v = find_vec(pre, nvec, idx);
  const RVec &r = V[v];
  if (!r.direct) return;
  const RDonor &d = D[r.donor];
  direct_item(in + r.io, out + r.io, d.a, d.an, d.dn, r.g, c2l, idx - pre[v]);
}

}  // namespace

struct l2c_gpu_ragged {
  size_t count = 0, total = 0, maxs = 0, dirs = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<l2c_gpu_plan *> donors;
  RVec *V = nullptr;
  RDonor *D = nullptr;
  long long *pre_all = nullptr;  // every prefix array, back to back
  long long *pre_coef = nullptr, *pre_leaf = nullptr, *pre_far = nullptr;
  long long *pre_rows = nullptr, tot_rows = 0;  // k_r_near_rows items
  std::vector<long long *> pre_up, pre_down;  // index d (1..Lmax-1), l (0..Lmax-2)
  long long tot_coef = 0, tot_leaf = 0, tot_far = 0;
  std::vector<long long> tot_up, tot_down;
  bool any_direct = false, any_fmm = false;
  int Lmax = 0;
  double *x = nullptr, *y = nullptr, *w = nullptr, *c = nullptr;
  double *st_in = nullptr, *st_out = nullptr;
  size_t cap_in = 0, cap_out = 0;
  size_t flops[2] = {0, 0};
  size_t launches = 0;
  std::mutex mu;
  // The band (and the direct-method vectors) on stream2 beside the far-field
  // chain, whose kernels then carry the device's greatest priority; joined
  // before leaf-down.  overlap / chain_prio: the plan's choices (L2C_OVERLAP,
  // L2C_CHAIN_PRIO); tuned_*: the autotuner's, per direction (-1: none).
  cudaStream_t stream2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // (the chain at its stream's priority by default: the band carries a ragged
  // list's step, 2000-vector list 17.18 -> 16.78 ms per L2C + C2L untuned)
  int overlap = 1, chain_prio = 0, prio_greatest = 0;
  int tuned_ov[2] = {-1, -1}, tuned_prio[2] = {-1, -1};
  double tuned_ms[2] = {0, 0}, tuned_ms_default[2] = {0, 0};
  bool autotune = false;
  // L2C_PLAN_PRECOMPUTE_NEAR: each donor keeps its dense band weights, which
  // the band of every vector with that leaf size reads (one DFMA per term)
  bool precompute = false;
};

namespace {

size_t ragged_launch(l2c_gpu_ragged *r, const double *in, double *out, size_t dir) {
  cudaStream_t st = r->stream;
  const int c2l = dir == 1, n = (int)r->count;
  const bool ov = r->any_fmm && (r->tuned_ov[dir] >= 0 ? r->tuned_ov[dir] : r->overlap) == 1;
  const bool hi = ov && (r->tuned_prio[dir] >= 0 ? r->tuned_prio[dir] : r->chain_prio) == 1;
  const LaunchOpt chain(false, hi ? r->prio_greatest : 0);
  cudaStream_t sb = ov ? r->stream2 : st;  // band and direct vectors
  if (r->any_fmm) {
    const double *x = in;  // L2C reads the caller's packed input directly
    if (c2l) {
      k_r_gather<<<blocks_for(r->tot_coef, 256), 256, 0, st>>>(in, r->x, r->V, r->pre_coef, n, 1);
      x = r->x;
      r->launches++;
    }
    if (ov) {
      CK(cudaEventRecord(r->ev_fork, st));
      CK(cudaStreamWaitEvent(r->stream2, r->ev_fork, 0));
    }
    (r->precompute ? k_r_near_rows<true> : k_r_near_rows<false>)<<<blocks_for(r->tot_rows, 256),
                                                                    256, 0, sb>>>(
        x, out, r->y, r->V, r->D, r->pre_rows, n, c2l);
    r->launches++;
    if (ov && r->any_direct) {  // other vectors' outputs: no order with the chain
      k_r_direct<<<blocks_for(r->tot_coef, 256), 256, 0, sb>>>(in, out, r->V, r->D, r->pre_coef,
                                                               n, c2l);
      r->launches++;
    }
    if (ov) CK(cudaEventRecord(r->ev_join, sb));
    launch_k(chain, k_r_leaf_up, blocks_for(r->tot_leaf, 288), 288, 0, st, x, r->w,
             (const RVec *)r->V, (const RDonor *)r->D, (const long long *)r->pre_leaf, n);
    r->launches++;
    for (int d = 1; d < r->Lmax; d++) {
      if (r->tot_up[d] == 0) continue;
      launch_k(chain, k_r_tree_up, blocks_for(r->tot_up[d], TREE_TILE), 32 * M, 0, st, r->w,
               (const RVec *)r->V, (const long long *)r->pre_up[d], n, d);
      r->launches++;
    }
    launch_k(chain, k_r_far, blocks_for(r->tot_far, 256), 256, 0, st, (const double *)r->w, r->c,
             (const RVec *)r->V, (const RDonor *)r->D, (const long long *)r->pre_far, n,
             (int)dir);
    r->launches++;
    for (int l = 0; l + 1 < r->Lmax; l++) {
      if (r->tot_down[l] == 0) continue;
      launch_k(chain, k_r_tree_down, blocks_for(r->tot_down[l], TREE_TILE), 32 * M, 0, st, r->c,
               (const RVec *)r->V, (const long long *)r->pre_down[l], n, l);
      r->launches++;
    }
    if (ov) CK(cudaStreamWaitEvent(st, r->ev_join, 0));
    k_r_leaf_down<<<blocks_for(r->tot_coef, 256), 256, 0, st>>>(r->c, r->y, out, r->V, r->D,
                                                                r->pre_coef, n, c2l);
    r->launches++;
  }
  if (r->any_direct && !ov) {
    k_r_direct<<<blocks_for(r->tot_coef, 256), 256, 0, st>>>(in, out, r->V, r->D, r->pre_coef, n,
                                                             c2l);
    r->launches++;
  }
  CK(cudaGetLastError());
  return 1;
}

}  // namespace

extern "C" {

void l2c_gpu_ragged_destroy(l2c_gpu_ragged *r) {
  if (!r) return;
  DeviceGuard dg(r->device);
  if (r->stream) cudaStreamSynchronize(r->stream);
  if (r->stream2) cudaStreamSynchronize(r->stream2);
  for (auto *d : r->donors) l2c_gpu_plan_destroy(d);
  void *bufs[] = {r->V, r->D, r->pre_all, r->x, r->y, r->w, r->c, r->st_in, r->st_out};
  for (void *b : bufs)
    if (b) cudaFree(b);
  if (r->ev_fork) cudaEventDestroy(r->ev_fork);
  if (r->ev_join) cudaEventDestroy(r->ev_join);
  if (r->stream2) cudaStreamDestroy(r->stream2);
  if (r->stream) cudaStreamDestroy(r->stream);
  delete r;
}

l2c_gpu_ragged *l2c_gpu_ragged_create(size_t count, const size_t *Ns, size_t maxs,
                                      size_t directions, unsigned flags) {
  g_err[0] = 0;
  if (count == 0 || !Ns || directions > 2) {
    set_err("ragged plan needs count > 0, lengths, and direction 0, 1 or 2");
    return nullptr;
  }
  l2c_gpu_ragged *r = new (std::nothrow) l2c_gpu_ragged();
  if (!r) return nullptr;
  auto fail = [&]() -> l2c_gpu_ragged * {
    l2c_gpu_ragged_destroy(r);
    return nullptr;
  };
#define RCK(call)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return fail();                                                                       \
    }                                                                                      \
  } while (0)
  r->count = count;
  r->maxs = maxs;
  r->dirs = directions;
  RCK(cudaGetDevice(&r->device));
  RCK(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
  RCK(cudaStreamCreateWithFlags(&r->stream2, cudaStreamNonBlocking));
  RCK(cudaEventCreateWithFlags(&r->ev_fork, cudaEventDisableTiming));
  RCK(cudaEventCreateWithFlags(&r->ev_join, cudaEventDisableTiming));
  {
    int least = 0, greatest = 0;
    RCK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    r->prio_greatest = greatest;
  }
  if (const char *env = std::getenv("L2C_OVERLAP")) r->overlap = env[0] == '1' ? 1 : 0;
  if (const char *env = std::getenv("L2C_CHAIN_PRIO")) r->chain_prio = env[0] == '1' ? 1 : 0;
  if (const char *env = std::getenv("L2C_AUTOTUNE")) r->autotune = env[0] == '1';
  r->precompute = (flags & L2C_PLAN_PRECOMPUTE_NEAR) != 0;
  // geometry of every vector; largest level count per leaf size s
  std::vector<size_t> L(count), S(count);
  std::vector<std::pair<size_t, size_t>> smax;  // (s, Lmax)
  size_t max_direct_N = 0;
  for (size_t v = 0; v < count; v++) {
    if (Ns[v] == 0) {
      set_err("vector %zu has length 0", v);
      return fail();
    }
    size_t sv = 0, nn = 0;
    L[v] = l2c_geometry(Ns[v], maxs, &sv, &nn);
    S[v] = sv;
    r->total += Ns[v];
    if (L[v] == 0) {
      max_direct_N = std::max(max_direct_N, Ns[v]);
      continue;
    }
    bool found = false;
    for (auto &e : smax)
      if (e.first == sv) {
        e.second = std::max(e.second, L[v]);
        found = true;
      }
    if (!found) smax.push_back({sv, L[v]});
  }
  // donors: one per s (A, T and Lambda tables), one direct-only table plan
  std::vector<RDonor> hD;
  std::vector<int> donor_of_s(smax.size());
  for (size_t k = 0; k < smax.size(); k++) {
    const size_t sv = smax[k].first, Lm = smax[k].second;
    l2c_gpu_plan *d = l2c_gpu_plan_create(sv << (Lm + 2), sv, directions,
                                          flags & L2C_PLAN_PRECOMPUTE_NEAR);
    if (!d) return fail();
    if (d->L != Lm || d->s != sv) {
      set_err("internal: donor geometry mismatch");
      l2c_gpu_plan_destroy(d);
      return fail();
    }
    r->donors.push_back(d);
    hD.push_back(RDonor{d->a, d->an, d->dn, d->T, {d->A[0], d->A[1]},
                        {d->Wtile[0], d->Wtile[1]}});
    r->Lmax = std::max(r->Lmax, (int)Lm);
  }
  int direct_donor = -1;
  if (max_direct_N > 0) {
    l2c_gpu_plan *d = l2c_gpu_plan_create(max_direct_N, 1, directions, L2C_PLAN_DIRECT_ONLY);
    if (!d) return fail();
    r->donors.push_back(d);
    hD.push_back(RDonor{d->a, d->an, d->dn, nullptr, {nullptr, nullptr}, {nullptr, nullptr}});
    direct_donor = (int)hD.size() - 1;
  }
  // descriptors and the prefix sums of each phase's work items
  std::vector<RVec> hV(count);
  const int Lmax = r->Lmax;
  std::vector<long long> pc(count + 1), pl(count + 1), pf(count + 1), pr(count + 1);
  std::vector<std::vector<long long>> pu(std::max(Lmax, 1), std::vector<long long>(count + 1)),
      pd(std::max(Lmax, 1), std::vector<long long>(count + 1));
  long long io = 0, wc = 0;
  for (size_t v = 0; v < count; v++) {
    RVec &e = hV[v];
    Geo &g = e.g;
    g.N = (long long)Ns[v];
    g.count = 1;
    g.dist = 0;
    g.stride = 1;
    g.L = (long long)L[v];
    e.io = io;
    e.wc = wc;
    e.direct = L[v] == 0;
    long long n_leaf = 0, n_far = 0;
    if (!e.direct) {
      g.s = (long long)S[v];
      g.h = 2 * g.s;
      g.nL = g.N / g.h;
      g.K = (long long)slots_at(L[v] - 1);
      g.slots = 2 * (long long)blocks_before(L[v]);
      g.leaf_base = 2 * (long long)blocks_before(L[v] - 1);
      size_t k = 0;
      while (smax[k].first != S[v]) k++;
      e.donor = (int)k;
      e.lshift = (int)(smax[k].second - L[v]);
      n_leaf = g.K * 2 * M;
      n_far = g.slots * M;  // 2 parities x N_b blocks x M
      wc += 2 * g.slots * M;
      r->any_fmm = true;
    } else {
      g.s = g.h = g.nL = g.K = g.slots = g.leaf_base = 0;
      e.donor = direct_donor;
      e.lshift = 0;
      r->any_direct = true;
    }
    pc[v + 1] = pc[v] + g.N;
    pr[v + 1] = pr[v] + (e.direct ? 0 : near_rows_items(g));
    pl[v + 1] = pl[v] + n_leaf;
    pf[v + 1] = pf[v] + n_far;
    for (int d = 1; d < Lmax; d++) {
      const long long l = (long long)L[v] - 1 - d;
      pu[d][v + 1] = pu[d][v] + ((!e.direct && l >= 0) ? 2 * (long long)slots_at((size_t)l) : 0);
    }
    for (int l = 0; l + 1 < Lmax; l++)
      pd[l][v + 1] = pd[l][v] + ((!e.direct && (long long)L[v] >= l + 2)
                                     ? 2 * (long long)slots_at((size_t)l) : 0);
    io += g.N;
    for (size_t d = 0; d < 2; d++)
      if (directions == d || directions == 2)
        r->flops[d] += ref_flops_geo(Ns[v], L[v], S[v], e.direct ? 0 : blocks_before(L[v]), d);
  }
  r->tot_coef = pc[count];
  r->tot_leaf = pl[count];
  r->tot_far = pf[count];
  r->tot_up.assign(std::max(Lmax, 1), 0);
  r->tot_down.assign(std::max(Lmax, 1), 0);
  const size_t nlev = (size_t)std::max(Lmax, 1);
  const size_t npre = (4 + 2 * nlev) * (count + 1);
  RCK(cudaMalloc(&r->pre_all, npre * sizeof(long long)));
  std::vector<long long> all;
  all.reserve(npre);
  auto push = [&](const std::vector<long long> &vv) { all.insert(all.end(), vv.begin(), vv.end()); };
  push(pc);
  push(pl);
  push(pf);
  for (size_t d = 0; d < nlev; d++) push(pu[d]);
  for (size_t l = 0; l < nlev; l++) push(pd[l]);
  push(pr);
  RCK(cudaMemcpy(r->pre_all, all.data(), npre * sizeof(long long), cudaMemcpyHostToDevice));
  r->pre_rows = r->pre_all + (3 + 2 * nlev) * (count + 1);
  r->tot_rows = pr[count];
  r->pre_coef = r->pre_all;
  r->pre_leaf = r->pre_all + (count + 1);
  r->pre_far = r->pre_all + 2 * (count + 1);
  r->pre_up.resize(nlev);
  r->pre_down.resize(nlev);
  for (size_t d = 0; d < nlev; d++) {
    r->pre_up[d] = r->pre_all + (3 + d) * (count + 1);
    r->tot_up[d] = pu[d][count];
  }
  for (size_t l = 0; l < nlev; l++) {
    r->pre_down[l] = r->pre_all + (3 + nlev + l) * (count + 1);
    r->tot_down[l] = pd[l][count];
  }
  RCK(cudaMalloc(&r->V, count * sizeof(RVec)));
  RCK(cudaMemcpy(r->V, hV.data(), count * sizeof(RVec), cudaMemcpyHostToDevice));
  RCK(cudaMalloc(&r->D, std::max<size_t>(hD.size(), 1) * sizeof(RDonor)));
  if (!hD.empty())
    RCK(cudaMemcpy(r->D, hD.data(), hD.size() * sizeof(RDonor), cudaMemcpyHostToDevice));
  RCK(cudaMalloc(&r->x, std::max<size_t>(r->total, 1) * sizeof(double)));
  RCK(cudaMalloc(&r->y, std::max<size_t>(r->total, 1) * sizeof(double)));
  RCK(cudaMalloc(&r->w, std::max<long long>(wc, 1) * sizeof(double)));
  RCK(cudaMalloc(&r->c, std::max<long long>(wc, 1) * sizeof(double)));
  return r;
#undef RCK
}

size_t l2c_gpu_ragged_total(const l2c_gpu_ragged *r) { return r ? r->total : 0; }

size_t l2c_gpu_ragged_flops(const l2c_gpu_ragged *r, size_t dir) {
  return (r && dir < 2) ? r->flops[dir] : 0;
}

void *l2c_gpu_ragged_stream(l2c_gpu_ragged *r) { return r ? (void *)r->stream : nullptr; }

size_t l2c_gpu_ragged_launch_count(const l2c_gpu_ragged *r) { return r ? r->launches : 0; }

}  // extern "C"

namespace {

// ms per ragged call with the band beside the chain or not (ov) and the chain
// at the greatest priority or not (pr), on device buffers: a warm-up call,
// then the best of three runs of two calls (CUDA events on the plan's stream,
// which stream2 joins).  < 0 on error.
double ragged_time(l2c_gpu_ragged *r, const double *in, double *out, size_t dir, int ov, int pr,
                   cudaEvent_t e0, cudaEvent_t e1) {
  r->tuned_ov[dir] = ov;
  r->tuned_prio[dir] = pr;
  bool ok = ragged_launch(r, in, out, dir) != 0;
  double best = -1.0;
  for (int rep = 0; rep < 3 && ok; rep++) {
    ok = cudaEventRecord(e0, r->stream) == cudaSuccess;
    for (int i = 0; i < 2 && ok; i++) ok = ragged_launch(r, in, out, dir) != 0;
    float ms = 0.f;
    ok = ok && cudaEventRecord(e1, r->stream) == cudaSuccess &&
         cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
    if (ok && (best < 0.0 || ms / 2.0 < best)) best = ms / 2.0;
  }
  return ok ? best : -1.0;
}

// The ragged list's autotuner: per direction, the band beside the chain or
// not and the chain's priority, timed on synthetic data of the list (the same
// bits under every choice).  Returns the tuned ms per call, 0 on error.
double ragged_tune(l2c_gpu_ragged *r, size_t dir) {
  double *din = nullptr, *dout = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double result = 0.0;
  const size_t n = r->total;
  if (cudaMalloc(&din, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dout, n * sizeof(double)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    set_err("autotuner: device allocation failed");
  } else {
    k_tune_fill<<<blocks_for((long long)n, 256), 256, 0, r->stream>>>(din, (long long)n);
    cudaMemsetAsync(dout, 0, n * sizeof(double), r->stream);
    int bo = r->overlap, bp = r->chain_prio;
    const double t_default = ragged_time(r, din, dout, dir, bo, bp, e0, e1);
    double best = t_default;
    const int cand[3][2] = {{0, 0}, {1, 0}, {1, 1}};
    for (int i = 0; i < 3 && best > 0.0 && r->any_fmm; i++) {
      if (cand[i][0] == r->overlap && (cand[i][0] == 0 || cand[i][1] == r->chain_prio)) continue;
      const double t = ragged_time(r, din, dout, dir, cand[i][0], cand[i][1], e0, e1);
      if (t < 0.0) {
        best = -1.0;
      } else if (t < 0.99 * best) {
        best = t;
        bo = cand[i][0];
        bp = cand[i][1];
      }
    }
    r->tuned_ov[dir] = bo;
    r->tuned_prio[dir] = bp;
    if (best > 0.0) {
      r->tuned_ms[dir] = best;
      r->tuned_ms_default[dir] = t_default;
      result = best;
    } else {
      r->tuned_ov[dir] = r->tuned_prio[dir] = -1;
      if (!g_err[0]) set_err("autotuner: a timed call failed");
    }
  }
  cudaStreamSynchronize(r->stream);
  cudaStreamSynchronize(r->stream2);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (din) cudaFree(din);
  if (dout) cudaFree(dout);
  return result;
}

}  // namespace

extern "C" {

double l2c_gpu_ragged_autotune(l2c_gpu_ragged *r, size_t dir) {
  g_err[0] = 0;
  if (!r || dir > 1 || !(r->dirs == dir || r->dirs == 2)) {
    set_err("null plan, or direction not planned");
    return 0.0;
  }
  std::lock_guard<std::mutex> lock(r->mu);
  DeviceGuard dg(r->device);
  return ragged_tune(r, dir);
}

int l2c_gpu_ragged_tuned_config(l2c_gpu_ragged *r, size_t dir, char *buf, size_t len,
                                double *ms) {
  if (!r || dir > 1) return -1;
  std::lock_guard<std::mutex> lock(r->mu);
  const bool t = r->tuned_ov[dir] >= 0;
  const int ov = t ? r->tuned_ov[dir] : r->overlap, pr = t ? r->tuned_prio[dir] : r->chain_prio;
  if (buf && len) snprintf(buf, len, "overlap=%d prio=%d", ov, pr);
  if (ms) {
    ms[0] = t ? r->tuned_ms[dir] : 0.0;
    ms[1] = t ? r->tuned_ms_default[dir] : 0.0;
  }
  return t ? 1 : 0;
}

size_t l2c_gpu_ragged_execute(l2c_gpu_ragged *r, const double *in, double *out, size_t dir,
                              unsigned flags) {
  g_err[0] = 0;
  if (!r || !in || !out) {
    set_err("null plan or array");
    return 0;
  }
  if (dir > 1 || !(r->dirs == dir || r->dirs == 2)) {
    set_err("direction %zu was not planned", dir);
    return 0;
  }
  std::lock_guard<std::mutex> lock(r->mu);
  DeviceGuard dg(r->device);
  if (r->autotune && r->any_fmm && r->tuned_ov[dir] < 0 && ragged_tune(r, dir) <= 0.0) return 0;
  const bool in_dev = is_device_ptr(in), out_dev = is_device_ptr(out);
  const size_t n = r->total;
  if (!in_dev) {
    if (!grow(&r->st_in, &r->cap_in, n)) return 0;
    CK(cudaMemcpyAsync(r->st_in, in, n * sizeof(double), cudaMemcpyHostToDevice, r->stream));
  }
  if (!out_dev) {
    if (!grow(&r->st_out, &r->cap_out, n)) return 0;
    CK(cudaMemcpyAsync(r->st_out, out, n * sizeof(double), cudaMemcpyHostToDevice, r->stream));
  }
  double *dout = out_dev ? out : r->st_out;
  if (!ragged_launch(r, in_dev ? in : r->st_in, dout, dir)) return 0;
  if (!out_dev)
    CK(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
  if (!(flags & L2C_EXEC_ASYNC) || !in_dev || !out_dev) CK(cudaStreamSynchronize(r->stream));
  return r->flops[dir];
}

int l2c_gpu_ragged_synchronize(l2c_gpu_ragged *r) {
  if (!r) return 1;
  DeviceGuard dg(r->device);
  if (cudaStreamSynchronize(r->stream) != cudaSuccess) {
    set_err("cudaStreamSynchronize failed");
    return 1;
  }
  return 0;
}

}  // extern "C"
