// Tensor-memory-accelerator (TMA) tile loads and shared-memory mbarriers, as
// inline PTX for sm_103a.  A CTA stages 2-D boxes of global vectors into shared
// memory with cp.async.bulk.tensor; one thread arms an mbarrier with the bytes
// to expect and issues the copies, every thread then waits on the barrier's
// phase (with a time limit) before reading the box.
#pragma once

#include <cstdint>
#include <cuda.h>  // CUtensorMap

#include "rkcu_device.cuh"

namespace rkcu {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make barrier initialisation visible to the async proxy (the TMA unit)
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Wait for the barrier phase with the given parity to complete, at most
// timeout_ns; on expiry record the error in the state and return false.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, DevState *st,
                                          unsigned long long timeout_ns, int site) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer_ns() - t0 > timeout_ns) {
      if (atomicCAS(&st->error, 0, 1) == 0) st->error_site = site;
      return false;
    }
  }
  return true;
}

// 2-D tile load: box of the tensor map at element coordinates (x, y) into
// shared memory at dst; completes bytes on the mbarrier.  x times the element
// size must be a multiple of 16 bytes; boxes may reach outside the tensor
// (those elements read as zero).
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// 1-D bulk copy of `bytes` (a multiple of 16) from global to shared memory,
// both addresses 16-byte aligned; completes bytes on the mbarrier.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// order this thread's generic-proxy global writes before later async-proxy
// (TMA) reads of the same memory
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

}  // namespace rkcu
