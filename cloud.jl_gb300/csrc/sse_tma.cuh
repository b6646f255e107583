// sse_tma.cuh -- bulk (TMA) copies of per-element slabs from global into
// shared memory, completed on an mbarrier.
//
// Every per-element array the kernels stage (states, metric terms, facet
// geometry, mass operators) is one contiguous slab, so one
// cp.async.bulk per slab, issued by one thread of the element's team, moves
// it through the copy engine while the team's threads stay free; the team
// then waits on the transaction count of one mbarrier.  A bulk copy needs
// 16-byte-aligned source and destination and a size that is a multiple of
// 16 bytes, and the slabs start anywhere: each copy covers the 16-byte
// aligned span around its slab (every device allocation that is staged this
// way carries 64 bytes of slack at its end, so the span never leaves the
// allocation), and the slab's first byte lands at the same offset modulo 16
// in the shared region, which therefore reserves 32 spare bytes.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sse {

// Shared-memory bytes a staged slab of `bytes` needs (span + alignment).
__host__ __device__ constexpr int staged_bytes(int bytes) { return bytes + 32; }

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make an mbarrier initialisation visible to the copy engine
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Wait for phase `parity` of the mbarrier with an iteration limit (each
// try_wait itself suspends for a bounded time); false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (int it = 0; it < (1 << 22); ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Prefetch `bytes` (a multiple of 16) of global memory from the 16-byte
// aligned address src into L2 through the copy engine; nothing waits on it.
__device__ __forceinline__ void prefetch_l2(const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Where a slab starting at global address src lands in a shared region
// (the region base is 16-byte aligned).
template <typename T>
__device__ __forceinline__ T *staged_ptr(void *region, const T *src) {
  return reinterpret_cast<T *>(static_cast<char *>(region) + (reinterpret_cast<uintptr_t>(src) & 15));
}

// Bytes moved by the bulk copy of a slab (its 16-byte-aligned span).
__device__ __forceinline__ uint32_t staged_span(const void *src, uint32_t bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(src);
  return (uint32_t)((((a + bytes) + 15) & ~(uintptr_t)15) - (a & ~(uintptr_t)15));
}

// Issue the bulk copy of a slab's aligned span into the region.
__device__ __forceinline__ void stage_slab(void *region, const void *src, uint32_t bytes, uint64_t *bar) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(src);
  bulk_copy_g2s(region, reinterpret_cast<const void *>(a & ~(uintptr_t)15), staged_span(src, bytes), bar);
}

}  // namespace sse
