// Entry points of the learned preconditioner used by the solver.
#pragma once

#include <cuda_runtime.h>

#include "sfx_learned.h"

namespace sfx_impl {

// z = s NN(r / s, features) on an nx x ny x nz node grid (device arrays)
int lnet_apply(sfx_lnet net, int nx, int ny, int nz, const float* r, const float* features, float* z, cudaStream_t s);
// SFX_ERR_TIMEOUT (once) if a convolution launched earlier gave up a bounded wait
int check_waits(sfx_lnet net);

}  // namespace sfx_impl
