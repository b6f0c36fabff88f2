// l2c_ozaki.cuh -- FP64-accurate small matrix products on BF16 tensor cores.
//
// Error-free splitting (Ozaki, Ogita, Oishi & Rump, "Error-free transformations
// of matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59 (2012)), arranged so that no FP64
// instruction is spent on the product:
//
//  * every row of the constant left factor P and every column of the data
//    factor Q shares a power-of-two scale 2^E with |x| < 2^E for all its entries;
//  * |x| 2^(56-E) is truncated to a 56-bit integer and cut into eight 7-bit
//    slices, x = sign * 2^E * sum_p s_p 2^(-7p), s_p in [0, 127] -- each slice is
//    an exact BF16 value;
//  * slice products with p + q <= OZ_DMAX are summed per diagonal d = p + q on
//    the tensor cores (mma.sync m16n8k16, BF16 in, FP32 accumulate); all
//    partial sums are integers below 2^24, so the accumulation is exact;
//  * the diagonal sums are combined exactly in 64-bit integer arithmetic,
//    T = sum_{d<=8} D_d 2^(7(8-d)) + floor(D_9 / 2^7), and T 2^(E_P + E_Q - 56) is
//    rounded once to a double by bit construction.
// Truncation of the operands and of the dropped diagonals bounds the error by
// about K 2^-53 |P|_row |Q|_col, the same order as FP64 summation.
#ifndef L2C_OZAKI_CUH
#define L2C_OZAKI_CUH

#include <cuda_bf16.h>

namespace l2c_oz {

constexpr int SLICES = 8;  // 7-bit slices
constexpr int FRAC = 56;   // fixed-point fraction bits = 7 * SLICES
constexpr int DMAX = 9;    // slice pairs p + q <= DMAX
constexpr int EXP_ZERO = -4000;

// Smallest E with |x| < 2^E (EXP_ZERO for zero and subnormals).
__host__ __device__ inline int exp_bound(double x) {
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
  const int ex = (int)((b >> 52) & 0x7FF);
  return ex == 0 ? EXP_ZERO : ex - 1022;
}

// Sign in bit 63, |x| 2^(56-E) truncated toward zero in bits 0..55 (|x| < 2^E).
__host__ __device__ inline unsigned long long fix56(double x, int E) {
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0 || E == EXP_ZERO) return 0;
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = 1075 + E - ex - FRAC;
  unsigned long long q;
  if (sh >= 64)
    q = 0;
  else if (sh <= 0)
    q = m << (-sh);
  else
    q = m >> sh;
  return q | (b & (1ull << 63));
}

// Signed slice p (1 = most significant) of a fix56 value.
__host__ __device__ inline float slice(unsigned long long f, int p) {
  const int v = (int)((f >> (FRAC - 7 * p)) & 127);
  return (f >> 63) ? -(float)v : (float)v;
}

__device__ __forceinline__ unsigned pack2(float lo, float hi) {
  __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned *>(&h);
}

// T 2^e rounded to nearest-even as a double (T a signed 64-bit integer).
__device__ __forceinline__ double to_double(long long T, int e) {
  if (T == 0) return 0.0;
  const unsigned long long neg = T < 0 ? 1ull : 0ull;
  unsigned long long a = neg ? (unsigned long long)(-T) : (unsigned long long)T;
  const int lz = __clzll((long long)a);
  a <<= lz;  // leading one at bit 63
  unsigned long long mant = a >> 11;
  const unsigned long long rest = a & 0x7FFull;
  if (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) mant++;
  int ex = 63 - lz + e;
  if (mant >> 53) {
    mant >>= 1;
    ex++;
  }
  if (ex < -1022) return 0.0;  // below the normal range: far under any output's ulp
  const unsigned long long bits =
      (neg << 63) | ((unsigned long long)(ex + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ void mma_bf16(float c[4], unsigned a0, unsigned a1, unsigned a2,
                                         unsigned a3, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// One warp: C = P Q for rows < MT*16 (rows >= mr are zero) and the warp's 8
// columns, FP64-accurate.
//   Ps  slices of P, element (p, r, k) at Ps[(p-1) * sstride + r * kld + k], k < kld
//       (entries with k >= K are never read: they are treated as zero)
//   Pe  per-row scale exponents of P
//   Qf  the 8 columns in fix56 form, Qf[c * qld + k], k < KT*16 (zero padded)
//   Qe  per-column scale exponents
// out[mt][e]: row mt*16 + (lane >> 2) + 8 (e >> 1), column 2 (lane & 3) + (e & 1).
template <int MT, int KT>
__device__ __forceinline__ void warp_tile(const __nv_bfloat16 *__restrict__ Ps, int sstride,
                                          int kld, int mr, int K, const int *__restrict__ Pe,
                                          const unsigned long long *Qf, int qld, const int *Qe,
                                          double out[MT][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  // B fragments of every slice: b0 = (k = 2t, 2t+1; col g), b1 = (k + 8)
  unsigned bf[SLICES][KT][2];
#pragma unroll
  for (int ks = 0; ks < KT; ks++) {
    const unsigned long long *c = Qf + g * qld + ks * 16 + 2 * t;
    const unsigned long long f0 = c[0], f1 = c[1], f8 = c[8], f9 = c[9];
#pragma unroll
    for (int q = 0; q < SLICES; q++) {
      bf[q][ks][0] = pack2(slice(f0, q + 1), slice(f1, q + 1));
      bf[q][ks][1] = pack2(slice(f8, q + 1), slice(f9, q + 1));
    }
  }
  long long T[MT][4];
#pragma unroll
  for (int mt = 0; mt < MT; mt++)
#pragma unroll
    for (int e = 0; e < 4; e++) T[mt][e] = 0;
#pragma unroll
  for (int d = 2; d <= DMAX; d++) {
    float acc[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[mt][e] = 0.f;
#pragma unroll
    for (int p = 1; p <= SLICES; p++) {
      const int q = d - p;
      if (q < 1 || q > SLICES) continue;
#pragma unroll
      for (int ks = 0; ks < KT; ks++) {
        const int k0 = ks * 16 + 2 * t;
#pragma unroll
        for (int mt = 0; mt < MT; mt++) {
          const int r0 = mt * 16 + g, r1 = r0 + 8;
          const __nv_bfloat16 *base = Ps + (p - 1) * sstride;
          unsigned a0 = 0, a1 = 0, a2 = 0, a3 = 0;
          if (r0 < mr) {
            if (k0 < K) a0 = *reinterpret_cast<const unsigned *>(base + r0 * kld + k0);
            if (k0 + 8 < K) a2 = *reinterpret_cast<const unsigned *>(base + r0 * kld + k0 + 8);
          }
          if (r1 < mr) {
            if (k0 < K) a1 = *reinterpret_cast<const unsigned *>(base + r1 * kld + k0);
            if (k0 + 8 < K) a3 = *reinterpret_cast<const unsigned *>(base + r1 * kld + k0 + 8);
          }
          mma_bf16(acc[mt], a0, a1, a2, a3, bf[q - 1][ks][0], bf[q - 1][ks][1]);
        }
      }
    }
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const long long v = (long long)__float2ll_rz(acc[mt][e]);
        T[mt][e] = d < DMAX ? (T[mt][e] << 7) + v : T[mt][e] + (v >> 7);
      }
  }
#pragma unroll
  for (int mt = 0; mt < MT; mt++)
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int r = mt * 16 + g + 8 * (e >> 1), c = 2 * t + (e & 1);
      out[mt][e] = r < mr ? to_double(T[mt][e], Pe[r] + Qe[c] - FRAC) : 0.0;
    }
}

}  // namespace l2c_oz

#endif
