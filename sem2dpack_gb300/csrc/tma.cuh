// tma.cuh -- bulk asynchronous copies (the TMA engine) and mbarriers in
// inline PTX for sm_103a.
//
// A batch of lattice rows is brought from global into shared memory with
// one cp.async.bulk per (row, plane); the copies signal an mbarrier with
// their byte counts (complete_tx) and the consumers wait on its phase.
// Every wait is bounded: after `limit` polls (kSpinLimit unless the step
// parameters give another) the caller gets `false` and reports an error
// instead of spinning forever.
#pragma once

#include <cstdint>

namespace sem2d {

constexpr int kSpinLimit = 1 << 22;  // polls of an mbarrier before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes initialised mbarriers visible to the async proxy
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one arrival that also announces `bytes` of transactions for this phase
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for the phase with the given parity to complete: at most
// `limit` polls (0: give up at once)
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int limit = kSpinLimit) {
  for (int k = 0; k < limit; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// global -> shared bulk copy of `bytes` (multiple of 16, both addresses
// 16-byte aligned), completion counted on `bar`
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

}  // namespace sem2d
