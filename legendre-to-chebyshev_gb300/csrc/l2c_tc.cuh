// l2c_tc.cuh -- fifth-generation tensor-core primitives (sm_100 family) in
// inline PTX: tensor-memory allocation, tcgen05.mma with operands in shared
// memory and the accumulator in tensor memory, its completion through an
// mbarrier, tensor-memory loads, the bulk asynchronous copy, and bounded
// mbarrier waits.  Written from the PTX ISA's description of these
// instructions.
//
// Operand layout used here: K-major without swizzling.  An 8-row x 16-byte
// "core matrix" (8 rows of 8 FP16 values) is 128 contiguous bytes, row r at
// byte 16 r.  A tile of R rows x 16 K values (one MMA's K) is R/8 x 2 core
// matrices: core (i, j) (rows 8i .. 8i+7, K values 8j .. 8j+7) at byte
// i * SBO + j * LBO, with LBO = 128 (the two K halves of a row group side by
// side) and SBO = 256 (row groups one after another): 16 R contiguous bytes.
#ifndef L2C_TC_CUH
#define L2C_TC_CUH

#include <cstdint>

namespace l2c_tc {

constexpr uint32_t CORE_LBO = 128;  // bytes between the two K halves of a row group
constexpr uint32_t CORE_SBO = 256;  // bytes between consecutive 8-row groups

// Byte offset of element (row, k) (k < 16) in a K-major no-swizzle tile.
__host__ __device__ inline uint32_t tile_offset(int row, int k) {
  return (uint32_t)(row >> 3) * CORE_SBO + (uint32_t)(k >> 3) * CORE_LBO +
         (uint32_t)(row & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading- and stride-
// dimension byte offsets (each >> 4), the fixed version bits 46 .. 48 =
// 0b001, base offset 0, relative leading-dimension mode, no swizzling.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP16 A and B (K-major), FP32 D,
// dense, M x N.
__host__ __device__ constexpr uint32_t idesc_f16_f32(int m, int n) {
  return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// ---- tensor memory --------------------------------------------------------
// Allocation by one whole warp; the base address is written to *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// Generic-proxy shared-memory writes made visible to the tensor core.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// D (tensor memory) = A B^T (+ D when acc): A and B from shared memory.
__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                       uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
// The mbarrier receives one arrival when every earlier tcgen05 operation of
// this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          smem_u32(bar))
      : "memory");
}

// Eight (four, two) consecutive 32-bit columns of the warp's 32 lanes (lane i
// of the warp reads tensor-memory lane (taddr >> 16) + i).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr)
               : "memory");
}
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, uint32_t (&r)[2]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(taddr)
               : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// ---- mbarriers and the bulk copy -------------------------------------------
__device__ __forceinline__ void bar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void bar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ bool bar_test(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Wait for the completion of the barrier's phase with this parity, for at
// most about `limit` SM clock cycles; false when the limit ran out.
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity,
                                         long long limit = 2000000000ll) {
  if (bar_test(bar, parity)) return true;
  const long long t0 = clock64();
  while (!bar_test(bar, parity)) {
    if (clock64() - t0 > limit) return false;
    __nanosleep(32);
  }
  return true;
}
// bytes (a multiple of 16) from global src to shared dst, completing a
// transaction count of that many bytes on bar (the caller's arrival states it).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes,
                                          uint64_t *bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
      "[%3];\n" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
#endif

}  // namespace l2c_tc

#endif
