// Entry points of the per-material kernel instantiations.
#pragma once

#include <cuda_runtime.h>

#include "form.hpp"

namespace sfx_impl {

int material_info(int material, int* components, int* nparams, int* state_doubles);

// mode: 0 residual, 1 residual committing state, 2 Jacobian action (FP64)
int launch_domain(const sfx_form_s& f, const DomainIntegral& di, int mode, const double* u, const double* du,
                  double* E, double t, cudaStream_t s);
int launch_domain_jvp_f32(const sfx_form_s& f, const DomainIntegral& di, const float* u, const float* du, float* E,
                          double t, cudaStream_t s);

}  // namespace sfx_impl
