// Bulk copies from global into shared memory through the Blackwell (sm_100+) TMA unit
// (cp.async.bulk, untiled), completed on an mbarrier, for staging a pair's hull vertices next to the
// warp that scans them.
//
// Rules this follows (PTX ISA, cp.async.bulk): source and destination 16-byte aligned, size a
// multiple of 16 bytes; only this GPU's own global memory is read, never with multicast. The
// caller copies the 16-byte-aligned body of a range and fetches its ragged head and tail (less
// than 16 bytes each) with plain loads, so no byte outside the range is read. Waits on the
// mbarrier are bounded: a wait that runs out of iterations returns false and the caller reports an
// error instead of spinning forever.
#pragma once
#include <cstdint>

namespace pg {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// mbarrier with `count` expected arrivals; made visible to the async proxy before any copy uses it.
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One arrival that also announces `bytes` of transactions the copies will complete.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory before later async-proxy
// writes (a buffer read by the warp is about to be refilled by a bulk copy).
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// dst (shared) <- src (global), `bytes` (multiple of 16; both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for the phase with the given parity to complete, at most `max_iters` polls (each poll may
// itself suspend for a hardware-chosen time). False when the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_iters) {
  for (uint32_t i = 0; i < max_iters; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

}  // namespace pg
