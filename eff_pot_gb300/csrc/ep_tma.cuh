// ep_tma.cuh - tensor-memory-access (TMA) copies and mbarriers for the
// stencil marches.
//
// A TMA copy moves a box of a 3-D tensor (described on the host by a
// CUtensorMap) from global into shared memory; one thread issues it, the copy
// engine fills shared memory and counts the bytes against an mbarrier, and the
// consumers wait on the barrier's phase.  Boxes that reach outside the tensor
// are filled with zeros.  Rules these copies follow: the box's innermost
// coordinate times the element size is a multiple of 16 bytes, the global
// strides are multiples of 16 bytes, every shared-memory destination is
// 128-byte aligned, and loads only (a load may start at a negative
// coordinate; it reads zeros there).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef EP_DEV
#define EP_DEV __device__ __forceinline__
#endif

EP_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

EP_DEV void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// Makes barrier initialisation visible to the copy engine.
EP_DEV void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
// Orders this thread's earlier shared-memory accesses (and those the block
// barrier made visible to it) before its later TMA copies.
EP_DEV void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// One arrival that also announces `bytes` of copies to come.
EP_DEV void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Waits for the phase with the given parity to complete; gives up after
// `limit` polls and returns false.
EP_DEV bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Box of a 3-D tensor at element coordinates (x, y, z) into shared memory.
EP_DEV void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
