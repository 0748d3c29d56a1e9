// Self-test of the bounded waits used by the bulk-copy kernels: one block
// waits on a shared-memory mbarrier that nothing arrives at, so the wait can
// only run out; the kernel records that in an error flag and returns.  No copy
// is in flight, so leaving the barrier incomplete is harmless.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "form.hpp"
#include "sfx.h"
#include "sfx/bulk.cuh"
#include "sfx/umma.cuh"

using namespace sfx_impl;

namespace {

__global__ void unsatisfiable_wait_kernel(uint32_t polls, int* __restrict__ err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    sfx::bulk::mbar_init(&bar, 1);
    sfx::bulk::fence_mbar_init();
  }
  __syncthreads();
  const bool done = sfx::bulk::mbar_wait(&bar, 0, polls);
  if (!done && threadIdx.x == 0) atomicExch(err, 1);
}

// Self-test of the tcgen05 path on one tile: D[128][N] = A[128][K] B[N][K]^T
// with BF16 operands staged in shared memory as K-major core matrices (K-half
// stride 128 B, row-group stride 256 B), the FP32 accumulator in TMEM and the
// result read back by tcgen05.ld.  Every wait is bounded; on a timeout the
// kernel records the error, waits once more (bounded) for the MMAs it issued
// and frees its TMEM before returning.
template <int N>
__global__ void __launch_bounds__(128) umma_tile_kernel(const __nv_bfloat16* __restrict__ A,
                                                        const __nv_bfloat16* __restrict__ B, int K,
                                                        float* __restrict__ D, int* __restrict__ err) {
  constexpr uint32_t NCOLS = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  constexpr uint32_t A_CHUNK = 128 * 32, B_CHUNK = N * 32;  // bytes per K-step of 16
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  const int nk = K / 16;
  unsigned char* sA = smem;
  unsigned char* sB = smem + size_t(nk) * A_CHUNK;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < 128 * K; i += blockDim.x) {
    const int r = i / K, k = i % K;
    *reinterpret_cast<__nv_bfloat16*>(sA + size_t(k / 16) * A_CHUNK + sfx::umma::kmajor_offset(r, k % 16, 128, 256)) =
        A[i];
  }
  for (int i = threadIdx.x; i < N * K; i += blockDim.x) {
    const int r = i / K, k = i % K;
    *reinterpret_cast<__nv_bfloat16*>(sB + size_t(k / 16) * B_CHUNK + sfx::umma::kmajor_offset(r, k % 16, 128, 256)) =
        B[i];
  }
  if (threadIdx.x == 0) {
    sfx::bulk::mbar_init(&bar, 1);
    sfx::bulk::fence_mbar_init();
  }
  if (warp == 0) {
    sfx::umma::tmem_alloc(&tmem_base, NCOLS);
    sfx::umma::tmem_relinquish();
  }
  sfx::bulk::fence_proxy_async_smem();  // the staged operands are read by the tensor core (async proxy)
  sfx::umma::fence_before_sync();
  __syncthreads();
  sfx::umma::fence_after_sync();
  const uint32_t tmem = tmem_base;
  if (threadIdx.x == 0) {
    constexpr uint32_t idesc = sfx::umma::idesc_bf16_f32(128, N);
    for (int kc = 0; kc < nk; kc++)
      sfx::umma::mma_bf16(tmem, sfx::umma::smem_desc(sA + size_t(kc) * A_CHUNK, 128, 256),
                          sfx::umma::smem_desc(sB + size_t(kc) * B_CHUNK, 128, 256), idesc, kc > 0);
    sfx::umma::commit(&bar);
  }
  const bool done = __syncthreads_and(sfx::bulk::mbar_wait(&bar, 0));
  sfx::umma::fence_after_sync();
  if (done) {
    const int row = 32 * warp + lane;
#pragma unroll
    for (int c = 0; c < N; c += 8) {
      float v[8];
      sfx::umma::ld_x8(tmem + (uint32_t(32 * warp) << 16) + uint32_t(c), v);
#pragma unroll
      for (int i = 0; i < 8; i++) D[row * N + c + i] = v[i];
    }
  } else {
    if (threadIdx.x == 0) atomicExch(err, 1);
    (void)sfx::bulk::mbar_wait(&bar, 0);  // the issued MMAs, bounded, before the TMEM is released
  }
  sfx::umma::fence_before_sync();
  __syncthreads();
  sfx::umma::fence_after_sync();
  if (warp == 0) sfx::umma::tmem_dealloc(tmem, NCOLS);
}

template <int N>
int umma_tile(const void* A, const void* B, int K, float* D, int* err) {
  const size_t smem = size_t(K / 16) * (128 * 32 + N * 32);
  SFX_CUDA_TRY(cudaFuncSetAttribute(umma_tile_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  umma_tile_kernel<N><<<1, 128, smem>>>(static_cast<const __nv_bfloat16*>(A), static_cast<const __nv_bfloat16*>(B),
                                        K, D, err);
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

}  // namespace

/* D = A B^T on one 128-row tile through tcgen05 (device pointers; A [128][K],
 * B [N][K] BF16 row-major, D [128][N] FP32); N in {16, 32, 48, 64, 128},
 * K a positive multiple of 16 up to 256.  SFX_ERR_TIMEOUT if the MMA did not
 * complete within the bounded wait. */
extern "C" int sfx_selftest_umma_tile(const void* A, const void* B, int N, int K, float* D) {
  if (!A || !B || !D) return fail(SFX_ERR_INVALID, "null pointer");
  if (K < 16 || K > 256 || K % 16) return fail(SFX_ERR_INVALID, "K must be a multiple of 16 in [16, 256]");
  MappedFlag flag;
  SFX_CUDA_TRY(flag.init());
  int rc = SFX_OK;
  switch (N) {
    case 16: rc = umma_tile<16>(A, B, K, D, flag.dev); break;
    case 32: rc = umma_tile<32>(A, B, K, D, flag.dev); break;
    case 48: rc = umma_tile<48>(A, B, K, D, flag.dev); break;
    case 64: rc = umma_tile<64>(A, B, K, D, flag.dev); break;
    case 128: rc = umma_tile<128>(A, B, K, D, flag.dev); break;
    default: return fail(SFX_ERR_INVALID, "N must be 16, 32, 48, 64 or 128");
  }
  if (rc) return rc;
  SFX_CUDA_TRY(cudaDeviceSynchronize());
  if (flag.raised()) return fail(SFX_ERR_TIMEOUT, "tensor-core MMA did not complete within the bounded wait");
  return SFX_OK;
}

extern "C" int sfx_selftest_bounded_wait(unsigned polls) {
  if (polls == 0) return fail(SFX_ERR_INVALID, "polls must be positive");
  MappedFlag flag;
  SFX_CUDA_TRY(flag.init());
  unsatisfiable_wait_kernel<<<1, 32>>>(polls, flag.dev);
  SFX_CUDA_TRY(cudaGetLastError());
  SFX_CUDA_TRY(cudaDeviceSynchronize());
  if (flag.raised()) return fail(SFX_ERR_TIMEOUT, "bounded wait expired (expected by this self-test)");
  return SFX_OK;
}
