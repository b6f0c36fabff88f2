// l2c_ozaki.cuh -- FP64-accurate small matrix products on FP16 tensor cores.
//
// Error-free splitting (Ozaki, Ogita, Oishi & Rump, "Error-free transformations
// of matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59 (2012)), arranged so that the product
// itself spends no FP64 instruction:
//
//  * every row of the constant factor P and every column of the data factor Q
//    shares a power-of-two scale 2^E with |x| < 2^E for all its entries;
//  * X = trunc(x 2^(53-E)) (|X| < 2^53) is written with six base-2^9 digits,
//    X = sum_p d_p 2^(9(6-p)), d_p = u_p - 256 where u_p are the bit fields of
//    Y = X + R, R = 256 sum_{k<6} 2^(9k) (0 <= Y < 2^55): nine bits for the five
//    low digits (d_p in [-256, 255]), ten for the top one (d_1 in [-256, 256]).
//    Every digit is an exact FP16 value, and two of them are formed at once as
//    the FP16 pair (1024 + u_a, 1024 + u_b) - (1280, 1280) from their bit fields;
//  * digit products with p + q <= DMAX = 7 are summed per diagonal d = p + q on
//    the tensor cores (mma.sync m16n8k16 / m16n8k8, FP16 in, FP32 accumulate).
//    A diagonal holds at most 6 digit pairs of magnitude <= 2^16, so for
//    K <= 40 terms every partial sum is an integer below 2^24 and the FP32
//    accumulation is exact;
//  * the diagonal sums are combined exactly in 64-bit integers,
//    T = sum_{d<=6} D_d 2^(9(6-d)) + floor(D_7 / 2^9), and the product is
//    T 2^(E_P + E_Q - 52), rounded once to a double by bit construction.
// The dropped diagonals (d >= 8) and the floor bound the error by a few units
// of 2^-53 |P|_row |Q|_col per product, the order of FP64 summation.
//
// Warp tile: 16 data columns (the mma "rows", A operand, sliced in registers)
// times NT x 8 outputs (the mma "columns", B operand: P transposed, pre-sliced
// at plan time into per-lane fragments held in shared memory).
#ifndef L2C_OZAKI_CUH
#define L2C_OZAKI_CUH

#include <cuda_fp16.h>

namespace l2c_oz {

constexpr int SLICES = 6;  // base-2^9 digits
constexpr int FRAC = 53;   // fixed-point fraction bits
constexpr int DMAX = 7;    // digit pairs p + q <= DMAX
constexpr int NDIAG = DMAX - 1;
constexpr int KMAX = 40;   // terms per exact accumulation
constexpr int EXP_ZERO = -4000;
constexpr long long RBAL = 0x20100804020100ll;  // 256 in every digit field

// Smallest E with |x| < 2^E (EXP_ZERO for zero and subnormals).
__host__ __device__ inline int exp_bound(double x) {
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
  const int ex = (int)((b >> 52) & 0x7FF);
  return ex == 0 ? EXP_ZERO : ex - 1022;
}

// Y = trunc(x 2^(FRAC-E)) + RBAL (|x| < 2^E; RBAL for zero).  Branch-free.
__host__ __device__ inline long long fixbal(double x, int E) {
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
  const int ex = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = 1075 + E - ex - FRAC;  // >= 0 when |x| < 2^E
  long long q = (long long)(m >> (sh < 63 ? sh : 63));
  q = (sh >= 64 || ex == 0 || E == EXP_ZERO) ? 0 : q;
  return (b >> 63) ? RBAL - q : RBAL + q;
}

// Digit p (1 = most significant) of Y as an exact float.
__host__ __device__ inline float digit_f(long long Y, int p) {
  if (p == 1) return (float)(int)((Y >> 45) & 1023) - 256.0f;
  return (float)(int)((Y >> (9 * (SLICES - p))) & 511) - 256.0f;
}

// FP16 bits of an integer of magnitude <= 2048 (exact).
__host__ __device__ inline unsigned half_bits(int v) {
  if (v == 0) return 0u;
  const unsigned s = v < 0 ? 0x8000u : 0u;
  unsigned a = (unsigned)(v < 0 ? -v : v);
  int e = 0;
  while ((a >> (e + 1)) != 0) e++;  // a in [2^e, 2^(e+1))
  return s | ((unsigned)(e + 15) << 10) | ((a << (10 - e)) & 0x3FFu);
}

#ifdef __CUDACC__
// Y split into two words: hi holds the fields of digits 1..3 (ten, nine and
// nine bits), lo those of digits 4..6.
struct Ysplit {
  unsigned hi, lo;
};
__device__ __forceinline__ Ysplit ysplit(long long Y) {
  return {(unsigned)((unsigned long long)Y >> 27), (unsigned)Y & 0x7FFFFFFu};
}
// Digit P of two values as one FP16 pair (value a in the low half): the two
// fields are placed in the mantissas of FP16 1024 + u (exact for u < 1024)
// and 1280 is subtracted from both halves.
template <int P>
__device__ __forceinline__ unsigned dig2(const Ysplit &a, const Ysplit &b) {
  constexpr int sh = P <= 3 ? 9 * (3 - P) : 9 * (6 - P);
  constexpr unsigned mask = P == 1 ? 0x3FFu : 0x1FFu;
  const unsigned wa = P <= 3 ? a.hi : a.lo, wb = P <= 3 ? b.hi : b.lo;
  const unsigned lo = (wa >> sh) & mask;
  const unsigned hi = (sh <= 16 ? wb << (16 - sh) : wb >> (sh - 16)) & (mask << 16);
  const unsigned w = lo | hi | 0x64006400u;
  const __half2 r = __hsub2(*reinterpret_cast<const __half2 *>(&w),
                            __halves2half2(__ushort_as_half(0x6500), __ushort_as_half(0x6500)));
  return *reinterpret_cast<const unsigned *>(&r);
}

__device__ __forceinline__ void mma16(float (&c)[4], const unsigned (&a)[4], unsigned b0,
                                      unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void mma8(float (&c)[4], unsigned a0, unsigned a1, unsigned b0) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(b0));
}

// Asynchronous global -> shared copies (bytes = 0 fills zeros).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes));
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }
#endif

// Fragment word of P^T for slice q (1-based), n-tile nt, k8-chunk c and lane
// (g = lane >> 2, t = lane & 3): P[8 nt + g][8 c + 2t .. 2t+1] as an FP16 pair.
// Chunks are interleaved in pairs (one 64-bit load per k16 step); an odd last
// chunk stands alone.  One matrix holds SLICES * NT * KC * 32 words.
__host__ __device__ inline int frag_index(int q, int nt, int c, int lane, int NT, int KC) {
  const int base = ((q - 1) * NT + nt) * KC * 32;
  if ((KC & 1) && c == KC - 1) return base + c * 32 + lane;
  return base + (c & ~1) * 32 + 2 * lane + (c & 1);
}

// Number of leading digit slices of a packed matrix that hold non-zero words
// (the later ones are zero for every row and k).
inline int used_slices(const unsigned *frag, int NT, int KC) {
  int used = 0;
  for (int q = 1; q <= SLICES; q++)
    for (int nt = 0; nt < NT; nt++)
      for (int c = 0; c < KC; c++)
        for (int lane = 0; lane < 32; lane++)
          if (frag[frag_index(q, nt, c, lane, NT, KC)] != 0u) used = q;
  return used;
}

#ifdef __CUDACC__
// T 2^e rounded to nearest-even as a double (T a signed 64-bit integer).
// Branch-free, so the independent outputs of a lane interleave.
__device__ __forceinline__ double to_double(long long T, int e) {
  const unsigned long long neg = (unsigned long long)T >> 63;
  const unsigned long long a = neg ? 0ull - (unsigned long long)T : (unsigned long long)T;
  const int lz = __clzll((long long)a);
  const unsigned long long n = a << (lz & 63);  // leading one at bit 63
  unsigned long long mant = n >> 11;
  const unsigned long long rest = n & 0x7FFull;
  mant += (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
  const unsigned long long carry = mant >> 53;
  mant >>= carry;
  const int ex = 63 - lz + e + (int)carry;
  const unsigned long long bits =
      (neg << 63) | ((unsigned long long)(ex + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull);
  // zero, and values below the normal range (far under any output's ulp), give 0
  return __longlong_as_double((a == 0 || ex < -1022) ? 0ll : (long long)bits);
}

// x truncated to a multiple of 2^e as an integer, when |x| < 2^(e+60) (the
// return value says whether it was).  Branch-free.
__device__ __forceinline__ bool to_fixed(double x, int e, long long &X) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = e + 1075 - ex;  // x = m 2^(ex-1075) = (m >> sh) 2^e; sh >= -7 when it fits
  unsigned long long q = sh >= 0 ? m >> (sh < 63 ? sh : 63) : m << ((-sh) & 63);
  q = (sh >= 64 || ex == 0) ? 0ull : q;
  X = (b >> 63) ? -(long long)q : (long long)q;
  return ex == 0 || ex - 1022 <= e + 60;
}

// Combined integer T of output (nt, e) from the NDIAG diagonal accumulators
// (each an exact integer below 2^24):
//   T = D0 2^36 + D1 2^27 + D2 2^18 + D3 2^9 + D4 + floor(D5 / 2^9),
// evaluated modulo 2^64 (T itself fits): three 32 x 32 -> 64-bit multiply-adds
// and the D0 term added to the high word in 32-bit arithmetic
// ((D0 2^4 mod 2^32) 2^32 = D0 2^36 mod 2^64) -- the same value as the
// nested form ((D0 2^9 + D1) 2^9 + ...) in half the integer instructions.
__device__ __forceinline__ long long combine6(float a0, float a1, float a2, float a3, float a4,
                                              float a5) {
  static_assert(NDIAG == 6, "the expansion below has six diagonals");
  const int d0 = __float2int_rn(a0), d1 = __float2int_rn(a1), d2 = __float2int_rn(a2);
  const int d3 = __float2int_rn(a3), d4 = __float2int_rn(a4), d5 = __float2int_rn(a5);
  long long t = (long long)(d4 + (d5 >> 9));
  t += (long long)d3 * (1 << 9);
  t += (long long)d2 * (1 << 18);
  t += (long long)d1 * (1 << 27);
  const unsigned hi = (unsigned)d0 << 4;
  return (long long)((unsigned long long)t + ((unsigned long long)hi << 32));
}
template <int NT>
__device__ __forceinline__ long long combine(const float (&acc)[NDIAG][NT][4], int nt, int e) {
  return combine6(acc[0][nt][e], acc[1][nt][e], acc[2][nt][e], acc[3][nt][e], acc[4][nt][e],
                  acc[5][nt][e]);
}

// The warp's 16 x (NT*8) tile over k8-chunks [C0, C1): acc[d-2][nt][.] = sum
// over k of the diagonal-d digit products, for the data columns (rows of the
// tile) in Ys.  C1 - C0 <= 5 (K <= 40) keeps the accumulation exact.
//   Ys : offset words Y of the 16 columns, column r at Ys[r * yld + k * ks],
//        k < 8 C1 (entries past the true K are RBAL, i.e. zero);
//   Pf : the fragment words of P^T (frag_index layout with KC chunks); its
//        slices past QMAX must be zero (they are not read).
// Output element (nt, e) of the lane is data column (lane >> 2) + 8 (e >> 1)
// and output row 8 nt + 2 (lane & 3) + (e & 1).
template <int NT, int KC, int C0 = 0, int C1 = KC, int QMAX = SLICES>
__device__ __forceinline__ void mma_tile(const unsigned *__restrict__ Pf, const long long *Ys,
                                         int yld, int ks, float (&acc)[NDIAG][NT][4]) {
  static_assert(C1 - C0 <= KMAX / 8, "accumulation would not be exact");
  // chunk pairs (2i, 2i+1) share one aligned 8-byte fragment load
  static_assert(C0 % 2 == 0, "a chunk range starts on a pair");
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int d = 0; d < NDIAG; d++)
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[d][nt][e] = 0.f;
  const long long *r0 = Ys + g * yld + 2 * t * ks, *r1 = r0 + 8 * yld;
#pragma unroll
  for (int c = C0; c < C1; c += 2) {
    if (c + 1 < C1) {
      const Ysplit y0 = ysplit(r0[(8 * c) * ks]), y1 = ysplit(r0[(8 * c + 1) * ks]);
      const Ysplit y2 = ysplit(r1[(8 * c) * ks]), y3 = ysplit(r1[(8 * c + 1) * ks]);
      const Ysplit y4 = ysplit(r0[(8 * c + 8) * ks]), y5 = ysplit(r0[(8 * c + 9) * ks]);
      const Ysplit y6 = ysplit(r1[(8 * c + 8) * ks]), y7 = ysplit(r1[(8 * c + 9) * ks]);
      unsigned a[SLICES][4];
#define L2C_OZ_SLICE(P)           \
  a[P - 1][0] = dig2<P>(y0, y1);  \
  a[P - 1][1] = dig2<P>(y2, y3);  \
  a[P - 1][2] = dig2<P>(y4, y5);  \
  a[P - 1][3] = dig2<P>(y6, y7);
      L2C_OZ_SLICE(1) L2C_OZ_SLICE(2) L2C_OZ_SLICE(3)
      L2C_OZ_SLICE(4) L2C_OZ_SLICE(5) L2C_OZ_SLICE(6)
#undef L2C_OZ_SLICE
#pragma unroll
      for (int q = 1; q <= QMAX; q++)
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
          const uint2 b =
              *reinterpret_cast<const uint2 *>(Pf + frag_index(q, nt, c, lane, NT, KC));
#pragma unroll
          for (int p = 1; p + q <= DMAX; p++) mma16(acc[p + q - 2][nt], a[p - 1], b.x, b.y);
        }
    } else {
      const Ysplit y0 = ysplit(r0[(8 * c) * ks]), y1 = ysplit(r0[(8 * c + 1) * ks]);
      const Ysplit y2 = ysplit(r1[(8 * c) * ks]), y3 = ysplit(r1[(8 * c + 1) * ks]);
      unsigned a[SLICES][2];
#define L2C_OZ_SLICE(P)           \
  a[P - 1][0] = dig2<P>(y0, y1);  \
  a[P - 1][1] = dig2<P>(y2, y3);
      L2C_OZ_SLICE(1) L2C_OZ_SLICE(2) L2C_OZ_SLICE(3)
      L2C_OZ_SLICE(4) L2C_OZ_SLICE(5) L2C_OZ_SLICE(6)
#undef L2C_OZ_SLICE
#pragma unroll
      for (int q = 1; q <= QMAX; q++)
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
          const unsigned b = Pf[frag_index(q, nt, c, lane, NT, KC)];
#pragma unroll
          for (int p = 1; p + q <= DMAX; p++) mma8(acc[p + q - 2][nt], a[p - 1][0], a[p - 1][1], b);
        }
    }
  }
}

// The FP16 digit fragments of a whole 16 x (8 KC) data tile, extracted once
// and kept in registers, for tiles multiplied by several constant factors (the
// two children of a downward transfer): a16 holds the k16 chunk pairs, a8 the
// trailing k8 chunk when KC is odd.  Same layout as mma_tile's per-chunk a.
template <int KC>
struct Digits {
  unsigned a16[KC / 2 > 0 ? KC / 2 : 1][SLICES][4];
  unsigned a8[SLICES][2];
};

template <int KC>
__device__ __forceinline__ void load_digits(const long long *Ys, int yld, int ks,
                                            Digits<KC> &D) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long long *r0 = Ys + g * yld + 2 * t * ks, *r1 = r0 + 8 * yld;
#pragma unroll
  for (int cp = 0; cp < KC / 2; cp++) {
    const int c = 2 * cp;
    const Ysplit y0 = ysplit(r0[(8 * c) * ks]), y1 = ysplit(r0[(8 * c + 1) * ks]);
    const Ysplit y2 = ysplit(r1[(8 * c) * ks]), y3 = ysplit(r1[(8 * c + 1) * ks]);
    const Ysplit y4 = ysplit(r0[(8 * c + 8) * ks]), y5 = ysplit(r0[(8 * c + 9) * ks]);
    const Ysplit y6 = ysplit(r1[(8 * c + 8) * ks]), y7 = ysplit(r1[(8 * c + 9) * ks]);
#define L2C_OZ_SLICE(P)                      \
  D.a16[cp][P - 1][0] = dig2<P>(y0, y1);     \
  D.a16[cp][P - 1][1] = dig2<P>(y2, y3);     \
  D.a16[cp][P - 1][2] = dig2<P>(y4, y5);     \
  D.a16[cp][P - 1][3] = dig2<P>(y6, y7);
    L2C_OZ_SLICE(1) L2C_OZ_SLICE(2) L2C_OZ_SLICE(3)
    L2C_OZ_SLICE(4) L2C_OZ_SLICE(5) L2C_OZ_SLICE(6)
#undef L2C_OZ_SLICE
  }
  if constexpr (KC & 1) {
    const int c = KC - 1;
    const Ysplit y0 = ysplit(r0[(8 * c) * ks]), y1 = ysplit(r0[(8 * c + 1) * ks]);
    const Ysplit y2 = ysplit(r1[(8 * c) * ks]), y3 = ysplit(r1[(8 * c + 1) * ks]);
#define L2C_OZ_SLICE(P)                \
  D.a8[P - 1][0] = dig2<P>(y0, y1);    \
  D.a8[P - 1][1] = dig2<P>(y2, y3);
    L2C_OZ_SLICE(1) L2C_OZ_SLICE(2) L2C_OZ_SLICE(3)
    L2C_OZ_SLICE(4) L2C_OZ_SLICE(5) L2C_OZ_SLICE(6)
#undef L2C_OZ_SLICE
  }
}

// One n-tile nt of a tile from cached digits: acc[d][.] = the diagonal-d sums
// over the KC chunks from chunk pair CP0 on (KC <= KMAX / 8 keeps them exact;
// CP0 > 0 skips pairs whose fragment words are zero for this n-tile), as
// mma_tile does for that n-tile.
template <int NT, int KC, int QMAX = SLICES, int CP0 = 0>
__device__ __forceinline__ void mma_nt(const unsigned *__restrict__ Pf, const Digits<KC> &D,
                                       int nt, float (&acc)[NDIAG][4]) {
  static_assert(KC <= KMAX / 8, "accumulation would not be exact");
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 0; d < NDIAG; d++)
#pragma unroll
    for (int e = 0; e < 4; e++) acc[d][e] = 0.f;
#pragma unroll
  for (int cp = CP0; cp < KC / 2; cp++) {
#pragma unroll
    for (int q = 1; q <= QMAX; q++) {
      const uint2 b = *reinterpret_cast<const uint2 *>(Pf + frag_index(q, nt, 2 * cp, lane, NT, KC));
#pragma unroll
      for (int p = 1; p + q <= DMAX; p++) mma16(acc[p + q - 2], D.a16[cp][p - 1], b.x, b.y);
    }
  }
  if constexpr (KC & 1) {
#pragma unroll
    for (int q = 1; q <= QMAX; q++) {
      const unsigned b = Pf[frag_index(q, nt, KC - 1, lane, NT, KC)];
#pragma unroll
      for (int p = 1; p + q <= DMAX; p++) mma8(acc[p + q - 2], D.a8[p - 1][0], D.a8[p - 1][1], b);
    }
  }
}

// combine() for one n-tile's accumulators.
__device__ __forceinline__ long long combine1(const float (&acc)[NDIAG][4], int e) {
  return combine6(acc[0][e], acc[1][e], acc[2][e], acc[3][e], acc[4][e], acc[5][e]);
}

// Column exponents and offset words of a staged tile, in place: Xs holds the
// raw doubles of 16 columns (column r at Xs[r * ld + k * ks], k < K); on
// return the same places hold the offset words Y, entries K <= k < KP hold
// RBAL, and Es[r] the column exponent.  Two lanes per column, each keeping its
// KP/2 entries in registers between the two passes.
template <int KP>
__device__ __forceinline__ void stage_fix(double *Xs, int ld, int ks, int K, int *Es) {
  constexpr int NV = (KP + 1) / 2;
  const int lane = threadIdx.x & 31, r = lane >> 1, h = lane & 1;
  double *row = Xs + r * ld;
  double v[NV];
  int e = EXP_ZERO;
#pragma unroll
  for (int i = 0; i < NV; i++) {
    const int k = 2 * i + h;
    v[i] = k < K ? row[k * ks] : 0.0;
    e = max(e, exp_bound(v[i]));
  }
  e = max(e, __shfl_xor_sync(0xffffffffu, e, 1));
  long long *yr = reinterpret_cast<long long *>(row);
#pragma unroll
  for (int i = 0; i < NV; i++) {
    const int k = 2 * i + h;
    if (k < KP) yr[k * ks] = k < K ? fixbal(v[i], e) : RBAL;
  }
  if (h == 0) Es[r] = e;
  __syncwarp();
}

// Column format of intermediate coefficient vectors: a column of values x_k
// is stored as integers V_k and one exponent E, x_k = V_k 2^(E - VBITS),
// |V_k| < 2^VBITS (E is arbitrary, and every V_k zero, for a zero column).
// Products leave their result in this form without rounding to double, and
// the next product re-normalises the column once (stage_cols).
constexpr int VBITS = 62;

// V 2^s (s >= 0) or floor(V 2^s) (s < 0), s clamped to [-63, 63].
__device__ __forceinline__ long long shift_s64(long long V, int s) {
  return s >= 0 ? V << (s < 63 ? s : 63) : V >> (-s < 63 ? -s : 63);
}

// In-place staging of 16 columns held in column format: column r of the tile
// is Xs[r * ld + k], k < K; entries k < K0 belong to a stored column with
// exponent Ea[r], entries k >= K0 to one with exponent Eb[r].  On return the
// same places hold the offset words Y of the column on a common scale with
// the largest entry at full precision (entries K <= k < KP hold RBAL) and
// Es[r] the column exponent (every |x_k| < 2^Es[r]).  Two lanes per column;
// each lane keeps its (KP+1)/2 entries in registers between the two passes.
template <int K, int K0, int KP>
__device__ __forceinline__ void stage_cols(long long *Xs, int ld, const int *Ea, const int *Eb,
                                           int *Es) {
  constexpr int NV = (KP + 1) / 2;
  const int lane = threadIdx.x & 31, r = lane >> 1, h = lane & 1;
  long long *row = Xs + r * ld;
  const int ea = Ea[r], eb = K0 < K ? Eb[r] : ea, ec = max(ea, eb);
  const int sa = -(ec - ea), sb = -(ec - eb);
  long long v[NV];
  unsigned long long m = 0;
#pragma unroll
  for (int i = 0; i < NV; i++) {
    const int k = 2 * i + h;
    v[i] = k < K ? shift_s64(row[k], k < K0 ? sa : sb) : 0;
    const unsigned long long a = v[i] < 0 ? 0ull - (unsigned long long)v[i] : (unsigned long long)v[i];
    m = a > m ? a : m;
  }
  const unsigned long long mo = __shfl_xor_sync(0xffffffffu, m, 1);
  m = mo > m ? mo : m;
  const int B = 64 - __clzll((long long)m);  // bits of the largest |V| (0 for a zero column)
  const int sh = FRAC - B;                   // in [-9, 53]
#pragma unroll
  for (int i = 0; i < NV; i++) {
    const int k = 2 * i + h;
    if (k < KP) row[k] = (k < K ? (sh >= 0 ? v[i] << sh : v[i] >> -sh) : 0) + RBAL;
  }
  if (h == 0) Es[r] = ec - VBITS + B;
  __syncwarp();
}
#endif

}  // namespace l2c_oz

#endif
