// sfx — 5th-generation tensor-core MMA (tcgen05) helpers for sm_103a, as
// inline PTX: tensor-memory (TMEM) allocation, shared-memory matrix and
// instruction descriptors, the single-thread MMA issue, its commit to an
// mbarrier, and the TMEM -> register loads of the epilogue.
//
// Operands are BF16, K-major, without swizzle: a tile is made of "core
// matrices" of 8 rows x 16 bytes (8 BF16) stored as 128 contiguous bytes; the
// descriptor gives the byte distance between core matrices adjacent along K
// (leading byte offset) and along M / N (stride byte offset).  The
// accumulator is FP32 in TMEM: row i of an M = 128 tile is TMEM lane i,
// column j is TMEM column (base + j).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "sfx/bulk.cuh"

namespace sfx {
namespace umma {

/// byte offset of element (row, k) of a K-major BF16 tile whose core
/// matrices are laid out with the given strides (row group stride `sbo`,
/// K-half stride `lbo`); k < 16 within one MMA K-step
__host__ __device__ constexpr uint32_t kmajor_offset(int row, int k, uint32_t lbo, uint32_t sbo) {
  return uint32_t(row >> 3) * sbo + uint32_t(k >> 3) * lbo + uint32_t(row & 7) * 16u + uint32_t(k & 7) * 2u;
}

/// shared-memory matrix descriptor (K-major, no swizzle, sm_100-family version 1)
__device__ inline uint64_t smem_desc(const void* base, uint32_t lbo_bytes, uint32_t sbo_bytes) {
  const uint64_t addr = bulk::smem_addr(base);
  uint64_t d = (addr >> 4) & 0x3FFFull;
  d |= uint64_t((lbo_bytes >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo_bytes >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;  // descriptor version; base offset 0, LBO mode 0, layout SWIZZLE_NONE
  return d;
}

/// instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32
/// accumulator, an M x N tile (M = 128 needs N a multiple of 16, 16..256)
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4)                       // accumulator format F32
         | (1u << 7)                     // A format BF16
         | (1u << 10)                    // B format BF16
         | (uint32_t(N >> 3) << 17)      // N / 8
         | (uint32_t(M >> 4) << 24);     // M / 16
}

/// TMEM allocation of `ncols` columns (a power of two >= 32) by one whole
/// warp; the base address is written to *dst (shared memory)
__device__ inline void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(bulk::smem_addr(dst)),
               "r"(ncols)
               : "memory");
}
__device__ inline void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ inline void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

/// D (TMEM) (+)= A B^T for one K-step of 16, issued by one thread
__device__ inline void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(uint32_t(accumulate))
      : "memory");
}

/// arrive once on `bar` when every MMA this thread issued so far has completed
__device__ inline void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bulk::smem_addr(bar))
               : "memory");
}

__device__ inline void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/// 8 consecutive FP32 columns of the calling warp's 32 TMEM lanes (lane
/// quarter = warp index % 4, encoded in taddr's upper half)
__device__ inline void ld_x8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace umma
}  // namespace sfx
