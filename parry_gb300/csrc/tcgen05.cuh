// Blackwell (sm_100+) fifth-generation tensor core operations for one CTA (cta_group::1), as inline
// PTX: shared-memory matrix descriptors, the f16-kind instruction descriptor, TMEM allocation,
// tcgen05.mma issue and commit, and tcgen05.ld of accumulators. Field layouts follow the PTX ISA
// (tcgen05 "Shared memory descriptor" and "Instruction descriptor" tables).
#pragma once
#include <cstdint>
#include "bulk_copy.cuh"

namespace pg {

// Matrix descriptor of a K-major operand without swizzling, in the canonical core-matrix layout:
// a core matrix is 8 rows x 16 bytes stored as 128 contiguous bytes; core matrices adjacent along
// K are `lbo` bytes apart, groups of 8 rows (along M or N) `sbo` bytes apart.
__device__ __forceinline__ uint64_t umma_desc_kmajor(const void* smem, uint32_t lbo, uint32_t sbo) {
  const uint64_t addr = smem_addr(smem);
  uint64_t d = 0;
  d |= (addr >> 4) & 0x3FFFull;                  // start address, bits 0-13
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;   // leading-dimension byte offset, bits 16-29
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;   // stride-dimension byte offset, bits 32-45
  d |= 1ull << 46;                               // descriptor version for tcgen05, bits 46-47
  return d;                                      // base offset 0, no swizzle (bits 61-63 = 0)
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 accumulation, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(uint32_t m, uint32_t n) {
  return (1u << 4)              // D format: F32
         | (1u << 7)            // A format: BF16
         | (1u << 10)           // B format: BF16
         | ((n >> 3) << 17)     // N >> 3, bits 17-22
         | ((m >> 4) << 24);    // M >> 4, bits 24-28
}

// D[tmem] (+)= A[smem] . B[smem]^T, issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}

// The mbarrier receives one arrival when every tcgen05.mma this thread issued before has completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void tc_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation of `ncols` columns (a power of two, at least 32) by one whole warp; the address
// is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive 32-bit accumulator columns of one TMEM lane per thread (the warp reads 32 lanes).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  // the registers pass through the wait, so no use of them can be scheduled before it
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]),
                 "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace pg
