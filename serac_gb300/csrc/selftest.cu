// Self-test of the bounded waits used by the bulk-copy kernels: one block
// waits on a shared-memory mbarrier that nothing arrives at, so the wait can
// only run out; the kernel records that in an error flag and returns.  No copy
// is in flight, so leaving the barrier incomplete is harmless.
#include <cuda_runtime.h>

#include "form.hpp"
#include "sfx.h"
#include "sfx/bulk.cuh"

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

}  // namespace

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
