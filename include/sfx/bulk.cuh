// sfx — bulk asynchronous copies (cp.async.bulk: the untiled TMA path, and
// cp.async.bulk.tensor: tiled loads through a tensor map) and
// shared-memory mbarriers for sm_90+ / sm_103a, as inline PTX.  Every wait is
// bounded: mbar_wait gives up after kMaxMbarPolls polls and reports failure,
// so a kernel can record an error and return instead of spinning forever.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sfx {
namespace bulk {

constexpr uint32_t kMaxMbarPolls = 1u << 22;

__device__ inline uint32_t smem_addr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

/// mbarrier with `count` expected arrivals per phase
__device__ inline void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
/// make barrier initialisation visible to the async proxy
__device__ inline void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
/// order this thread's earlier generic-proxy shared-memory accesses before later async-proxy ones
__device__ inline void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
/// one arrival that also expects `bytes` of transaction (the bulk copy that follows)
__device__ inline void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
/// global -> shared bulk copy completing on `bar`; dst, src 16-byte aligned, bytes a multiple of 16
__device__ inline void copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
/// tiled tensor load (cp.async.bulk.tensor, 5-D, the TMA tile path) of the
/// box at coordinates (c0..c4) of the tensor map `map` (a __grid_constant__
/// kernel parameter or global memory) into shared memory, completing on
/// `bar`.  c0 * element size must be a multiple of 16 bytes; the other
/// coordinates may lie outside the tensor (those elements read zero).
__device__ inline void tma_load_5d(void* dst, const void* map, int c0, int c1, int c2, int c3, int c4,
                                   uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_addr(bar))
      : "memory");
}
/// one poll: whether the phase of parity `parity` has completed
__device__ inline bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
/// bounded wait for the phase of parity `parity`; false if it did not complete
/// within `polls` polls
__device__ inline bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t polls = kMaxMbarPolls) {
  for (uint32_t k = 0; k < polls; k++)
    if (mbar_test(bar, parity)) return true;
  return false;
}

}  // namespace bulk
}  // namespace sfx
