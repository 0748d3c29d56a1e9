/*
 * sfx — learned multilevel preconditioner (C ABI).  No counterpart in serac:
 * a small 3-D convolutional network on the node grid of a structured H1
 * mesh that maps a residual to an approximate Newton correction, trained on
 * (residual, correction) pairs harvested from the plain solver, and used
 * inside flexible GMRES with a Jacobi-Chebyshev fallback.
 *
 * Network (fixed architecture, ~290k parameters, BF16 activations and
 * weights on the tensor cores, FP32 accumulation, FP32 master weights):
 *   input 16 channels: residual / s (3), node feature (log modulus),
 *   Dirichlet mask, zeros; s = root-mean-square of the residual
 *   level 0: conv 16->16, conv 16->16          (skip 0)
 *   level 1: restrict, conv 16->32, conv 32->32 (skip 1)
 *   level 2: restrict, conv 32->48, conv 48->48 (skip 2)
 *   level 3: restrict, conv 48->48
 *   up: prolong + skip 2, conv 48->32; prolong + skip 1, conv 32->16;
 *       prolong + skip 0, conv 16->16; output conv 16->16 (first 3 channels)
 * all 3x3x3 convolutions with zero padding and ReLU except the output one;
 * restriction = full weighting (P^T / 8), prolongation P = trilinear.
 * Grids nest as 2m+1 -> m+1 nodes per direction, so the node grid of an
 * order-2 structured mesh with n elements per direction ((2n+1)^3) works for
 * n divisible by 8.
 *
 * Vectors are byNODES on the node grid (component * N + node, node
 * x-fastest), features are [2][N] (log modulus, Dirichlet mask).
 */
#ifndef SFX_LEARNED_H
#define SFX_LEARNED_H

#include <stdint.h>

#include "sfx.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sfx_lnet_s* sfx_lnet;

/* He-initialised network from a seed (deterministic host PRNG). */
int sfx_lnet_create(uint64_t seed, sfx_lnet* out);
int sfx_lnet_destroy(sfx_lnet net);
int sfx_lnet_num_params(sfx_lnet net, int64_t* n);
/* Parameter vector: for each convolution in the order above, W[cout][27][cin] then b[cout]. */
int sfx_lnet_get_params(sfx_lnet net, float* host, int64_t n);
int sfx_lnet_set_params(sfx_lnet net, const float* host, int64_t n);

/* z = s NN(r / s, features) with z = 0 on masked nodes (device arrays). */
int sfx_lnet_apply(sfx_lnet net, int nx, int ny, int nz, const float* r, const float* features, float* z,
                   void* stream);

/* Loss and parameter gradient for one sample without an update (host
 * outputs; for gradient checks).  loss = sum over unmasked nodes of
 * |NN(r/s) - t/s|^2 / sum |t/s|^2 with t the target correction. */
int sfx_lnet_gradient(sfx_lnet net, int nx, int ny, int nz, const float* r, const float* target,
                      const float* features, float* loss, float* grad_host, void* stream);

/* One Adam step (lr, beta1 0.9, beta2 0.999) on the mean gradient of a batch
 * of samples ([batch][3N] residuals and targets, [batch][2N] features, device). */
int sfx_lnet_train_step(sfx_lnet net, int nx, int ny, int nz, int batch, const float* r, const float* target,
                        const float* features, float lr, float* mean_loss, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SFX_LEARNED_H */
