// tma.cuh -- inline-PTX helpers for 1-D bulk asynchronous copies (TMA) into
// shared memory, completed through an mbarrier transaction count.
//
//   thread 0:  mbar_init(bar, 1); fence; __syncthreads()
//              mbar_expect_tx(bar, total_bytes); bulk_g2s(dst, src, bytes, bar) ...
//   all:       mbar_wait_bounded(bar, phase, err)   -- never spins unbounded
//
// A bulk copy needs 16-byte aligned source and destination and a size that is
// a multiple of 16 bytes; callers check this before choosing this path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nekgpu {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Make the initialised barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// The same copy with an L2 eviction-priority policy for the source lines.
__device__ __forceinline__ void bulk_g2s_hint(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1], %2, [%3], %4;" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Each try_wait suspends for a hardware-chosen interval; 2^22 tries is
// seconds, far beyond any copy.  On expiry the block records an error in
// *err and waits once more, again bounded, so that no copy is still writing
// into shared memory when the block leaves.
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, int* err) {
  for (uint32_t it = 0; it < kWaitLimit; ++it)
    if (mbar_try_wait(bar, phase)) return true;
  if (err) atomicOr(err, 1);
  for (uint32_t it = 0; it < kWaitLimit; ++it)
    if (mbar_try_wait(bar, phase)) break;
  return false;
}

}  // namespace nekgpu
