// Learned multilevel preconditioner: network state, forward / backward
// orchestration and Adam (the architecture is described in include/sfx_learned.h).
// Every pass runs on a batch of samples at once (blockIdx.y of each kernel
// selects the sample); per-sample scales and losses stay on the device, so a
// training step synchronises with the host once (to report the loss) and an
// inference pass not at all.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <random>
#include <string>
#include <tuple>
#include <vector>

#include "form.hpp"
#include "learned_internal.hpp"
#include "sfx.h"
#include "sfx/nn.cuh"
#include "sfx_learned.h"

using namespace sfx_impl;
using sfx::nn::Grid3;
using bf16 = __nv_bfloat16;

namespace {

#define SFX_TRY(call)                  \
  do {                                 \
    if (int rc_ = (call)) return rc_;  \
  } while (0)

inline unsigned nb(int64_t n, int b = 256) { return unsigned((n + b - 1) / b); }
inline dim3 grid2(int64_t n, int batch, int b = 256) { return dim3(nb(n, b), unsigned(batch)); }

// ----------------------------------------------------------- small kernels
__global__ void f32_to_bf16(const float* __restrict__ a, bf16* __restrict__ b, int64_t n) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16(a[i]);
}
// g_pre = g * (y > 0) (ReLU backward), as fp32 and bf16; relu = false copies
__global__ void act_bwd(const float* __restrict__ g, const bf16* __restrict__ y, bool relu, float* __restrict__ gp,
                        bf16* __restrict__ gp16, int64_t n) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = (!relu || __bfloat162float(y[i]) > 0.f) ? g[i] : 0.f;
  gp[i] = v;
  gp16[i] = __float2bfloat16(v);
}
__global__ void add_into(const float* __restrict__ a, float* __restrict__ b, int64_t n) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] += a[i];
}
// d = float(a) + float(b) ; and its bf16 copy
__global__ void add_bf16_into(const bf16* __restrict__ a, float* __restrict__ d, bf16* __restrict__ d16, int64_t n) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = d[i] + __bfloat162float(a[i]);
  d[i] = v;
  d16[i] = __float2bfloat16(v);
}
// x0[b][n][0..15] = {r/s_b (3), feature, constraint, 0...}
__global__ void pack_input(const float* __restrict__ r, const float* __restrict__ feat, int64_t N,
                           const float* __restrict__ scale, bf16* __restrict__ x0) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int64_t b = blockIdx.y;
  r += b * 3 * N;
  feat += b * 2 * N;
  x0 += b * N * 16;
  const float inv_s = 1.f / scale[b];
  float v[16] = {};
  for (int c = 0; c < 3; c++) v[c] = r[c * N + n] * inv_s;
  v[3] = feat[n];
  v[4] = feat[N + n];
  for (int c = 0; c < 16; c++) x0[n * 16 + c] = __float2bfloat16(v[c]);
}
// z[b][c N + n] = s_b out[b][n][c] (0 on masked nodes)
__global__ void unpack_output(const float* __restrict__ out, const float* __restrict__ feat, int64_t N,
                              const float* __restrict__ scale, float* __restrict__ z) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int64_t b = blockIdx.y;
  out += b * N * 16;
  feat += b * 2 * N;
  z += b * 3 * N;
  const bool masked = feat[N + n] > 0.5f;
  const float s = scale[b];
  for (int c = 0; c < 3; c++) z[c * N + n] = masked ? 0.f : s * out[n * 16 + c];
}
// squared error per node and gradient of loss_b = sum |out - t/s_b|^2 / tt_b
__global__ void loss_grad(const float* __restrict__ out, const float* __restrict__ t, const float* __restrict__ feat,
                          int64_t N, const float* __restrict__ scale, const float* __restrict__ inv_tt,
                          float* __restrict__ g, float* __restrict__ err) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int64_t b = blockIdx.y;
  out += b * N * 16;
  t += b * 3 * N;
  feat += b * 2 * N;
  g += b * N * 16;
  err += b * N;
  const bool masked = feat[N + n] > 0.5f;
  const float inv_s = 1.f / scale[b], itt = inv_tt[b];
  float e = 0.f;
  for (int c = 0; c < 16; c++) {
    float d = 0.f;
    if (c < 3 && !masked) d = out[n * 16 + c] - t[c * N + n] * inv_s;
    g[n * 16 + c] = 2.f * d * itt;
    e += d * d;
  }
  err[n] = e;
}
// |t/s_b|^2 per unmasked node
__global__ void target_sq(const float* __restrict__ t, const float* __restrict__ feat, int64_t N,
                          const float* __restrict__ scale, float* __restrict__ out) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int64_t b = blockIdx.y;
  t += b * 3 * N;
  feat += b * 2 * N;
  const float inv_s = 1.f / scale[b];
  float e = 0.f;
  if (feat[N + n] <= 0.5f)
    for (int c = 0; c < 3; c++) {
      const float v = t[c * N + n] * inv_s;
      e += v * v;
    }
  out[b * N + n] = e;
}
__global__ void square(const float* __restrict__ a, float* __restrict__ b, int64_t n) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i] * a[i];
}
// out[b] = sum of a[b * len .. (b + 1) * len) in double, fixed order, in two
// passes: block (g, b) sums chunk g of segment b into part[b][g]; then one
// block per segment sums its kSegChunks partials
constexpr int kSegChunks = 64;
__global__ void __launch_bounds__(256) segment_partials(const float* __restrict__ a, int64_t len,
                                                        double* __restrict__ part) {
  __shared__ double sh[256];
  const int64_t chunk = (len + kSegChunks - 1) / kSegChunks;
  const int64_t b0 = int64_t(blockIdx.x) * chunk, b1 = b0 + chunk < len ? b0 + chunk : len;
  const float* seg = a + int64_t(blockIdx.y) * len;
  double acc = 0.0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += 256) acc += seg[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[int64_t(blockIdx.y) * kSegChunks + blockIdx.x] = sh[0];
}
__global__ void segment_finish(const double* __restrict__ part, float* __restrict__ out) {
  __shared__ double sh[kSegChunks];
  sh[threadIdx.x] = part[int64_t(blockIdx.x) * kSegChunks + threadIdx.x];
  __syncthreads();
  for (int s = kSegChunks / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = float(sh[0]);
}
void segment_sums(const float* a, int64_t len, int nseg, double* part, float* out, cudaStream_t s) {
  segment_partials<<<dim3(kSegChunks, unsigned(nseg)), 256, 0, s>>>(a, len, part);
  segment_finish<<<unsigned(nseg), kSegChunks, 0, s>>>(part, out);
}
// scale[b] = RMS of the residual (1 for a zero residual)
__global__ void make_scale(const float* __restrict__ ss, int64_t len, int batch, float* __restrict__ scale) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) scale[b] = ss[b] > 0.f ? sqrtf(ss[b] / float(len)) : 1.f;
}
__global__ void make_inverse(const float* __restrict__ a, int batch, float* __restrict__ inv) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) inv[b] = a[b] > 0.f ? 1.f / a[b] : 0.f;
}
__global__ void adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                     int64_t n, float lr, float b1, float b2, float c1, float c2, float eps, float gscale) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] * gscale;
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
}

// --------------------------------------------------------- conv dispatch
#define SFX_PAIRS(X) X(16, 16) X(16, 32) X(32, 32) X(32, 48) X(48, 48) X(48, 32) X(32, 16)

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (no link-time dependency on libcuda)
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    looked_up = true;
  }
  return fn;
}

// tensor map of `batch` activation volumes [z][y][x][C] (BF16) with the brick
// convolution's box: 8 channels x (8 + 2) x (16 + 2) x (BZ + 2) nodes x 1 sample
int activation_map(CUtensorMap* map, const bf16* x, int C, Grid3 g, int batch, int bz) {
  auto fn = encode_tiled();
  if (!fn) return fail(SFX_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint64_t dims[5] = {cuuint64_t(C), cuuint64_t(g.nx), cuuint64_t(g.ny), cuuint64_t(g.nz), cuuint64_t(batch)};
  const cuuint64_t row = cuuint64_t(C) * 2;
  const cuuint64_t strides[4] = {row, row * g.nx, row * g.nx * g.ny, row * g.nx * g.ny * g.nz};
  const cuuint32_t box[5] = {8, 10, 18, cuuint32_t(bz + 2), 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16*>(x), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(SFX_ERR_CUDA, "cuTensorMapEncodeTiled failed for an activation volume");
  return SFX_OK;
}

// the tensor-core (tcgen05) brick convolution: one block per 8 x 16 x BZ
// output nodes and sample (the dynamic shared-memory limit is raised once per
// instantiation)
template <int CI, int CO, int ACT>
int launch_conv(Grid3 g, int batch, const bf16* x, const bf16* W, const float* b, bf16* y, float* y32, int* err,
                cudaStream_t s) {
  using L = sfx::nn::BrickConvSmem<CI, CO>;
  static bool configured = false;
  if (!configured) {
    SFX_CUDA_TRY(cudaFuncSetAttribute(sfx::nn::conv3_fwd_brick<CI, CO, ACT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, int(L::bytes)));
    configured = true;
  }
  CUtensorMap map;
  if (int rc = activation_map(&map, x, CI, g, batch, L::BZ)) return rc;
  const int64_t bricks = int64_t((g.nx + 7) / 8) * ((g.ny + 15) / 16) * ((g.nz + L::BZ - 1) / L::BZ);
  const dim3 blocks{unsigned(bricks), unsigned(batch)};
  sfx::nn::conv3_fwd_brick<CI, CO, ACT><<<blocks, 128, L::bytes, s>>>(map, g, W, b, y, y32, err);
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

int conv_fwd(int ci, int co, bool relu, Grid3 g, int batch, const bf16* x, const bf16* W, const float* b, bf16* y,
             float* y32, int* err, cudaStream_t s) {
#define SFX_CONV(CI, CO)                                                                       \
  if (ci == CI && co == CO) {                                                                  \
    if (relu) return launch_conv<CI, CO, sfx::nn::ACT_RELU>(g, batch, x, W, b, y, y32, err, s); \
    return launch_conv<CI, CO, sfx::nn::ACT_NONE>(g, batch, x, W, b, y, y32, err, s);           \
  }
  SFX_PAIRS(SFX_CONV)
#undef SFX_CONV
  return fail(SFX_ERR_UNSUPPORTED, "no convolution for these channel counts");
}
// blocks of the weight-gradient kernel for a grid and batch (at most 4 per SM)
int wgrad_blocks(Grid3 g, int batch) {
  const int64_t nchunks = (g.nodes() + sfx::nn::kWgradChunk - 1) / sfx::nn::kWgradChunk * batch;
  return int(std::min<int64_t>(nchunks, 4 * 152));
}
void conv_wgrad(int ci, int co, Grid3 g, int batch, const bf16* x, const bf16* dy, float* part, cudaStream_t s) {
#define SFX_WG(CI, CO)                                                                              \
  if (ci == CI && co == CO) {                                                                       \
    sfx::nn::conv3_wgrad_mma<CI, CO><<<wgrad_blocks(g, batch), 128, 0, s>>>(g, batch, x, dy, part); \
    return;                                                                                         \
  }
  SFX_PAIRS(SFX_WG)
#undef SFX_WG
}
void flip(int ci, int co, const bf16* W, bf16* Wt, cudaStream_t s) {
#define SFX_FL(CI, CO)                                                              \
  if (ci == CI && co == CO) {                                                       \
    sfx::nn::flip_weights<CI, CO><<<nb(CI * 27 * CO), 256, 0, s>>>(W, Wt);          \
    return;                                                                         \
  }
  SFX_PAIRS(SFX_FL)
#undef SFX_FL
}
void pack(int ci, int co, const bf16* W, bf16* Wp, cudaStream_t s) {
#define SFX_PK(CI, CO)                                                                      \
  if (ci == CI && co == CO) {                                                               \
    sfx::nn::pack_brick_weights<CI, CO><<<nb(CO * 27 * CI / 8), 256, 0, s>>>(W, Wp);        \
    return;                                                                                 \
  }
  SFX_PAIRS(SFX_PK)
#undef SFX_PK
}
void bias_grad(int co, const float* dy, int64_t rows, float* db, cudaStream_t s) {
  if (co == 16) sfx::nn::bias_grad<16><<<16, 256, 0, s>>>(dy, rows, db);
  else if (co == 32) sfx::nn::bias_grad<32><<<32, 256, 0, s>>>(dy, rows, db);
  else sfx::nn::bias_grad<48><<<48, 256, 0, s>>>(dy, rows, db);
}

struct Conv {
  int ci, co;
  bool relu;
  int64_t off;  // offset of W in the parameter vector (b follows)
  int64_t nw() const { return int64_t(co) * 27 * ci; }
};

enum { A0, B0L, A1, B1L, A2, B2L, A3, U2, U1, U0, OUTL, NLAYERS };
constexpr int kLevel[NLAYERS] = {0, 0, 1, 1, 2, 2, 3, 2, 1, 0, 0};  // grid level of each layer

// activations and gradients of up to `cap` samples on one node grid
struct Work {
  Grid3 g[4];
  int cap = 0;
  DeviceBuf<bf16> X0, A0b, B0b, C1, A1b, B1b, C2, A2b, B2b, C3, A3b, D2b, E2, D1b, E1, D0b, E0;
  DeviceBuf<float> D2, D1, D0, OUT;
  DeviceBuf<float> gOUT, gE0, gD0, gE1, gD1, gE2, gD2, gA3, gC3, gB2, gA2, gC2, gB1, gA1, gC1, gB0, gA0, gpre, tmpf;
  DeviceBuf<bf16> gpre16;
  DeviceBuf<float> part, red, err;
  DeviceBuf<float> ss, scale, tt, inv_tt, esum;  // per sample
  DeviceBuf<double> seg;                         // partial sums of segment_sums [sample][kSegChunks]
};

}  // namespace

struct sfx_lnet_s {
  sfx_impl::MappedFlag wait_error;  // set by a convolution whose bounded wait expired
  Conv layers[NLAYERS];
  int64_t nparams = 0;
  DeviceBuf<float> P, G, M, V;  // master parameters, gradient, Adam moments
  DeviceBuf<bf16> W16[NLAYERS], Wt16[NLAYERS];    // [co][tap][ci], and flipped for the data gradient
  DeviceBuf<bf16> Wp16[NLAYERS], Wtp16[NLAYERS];  // the same packed for the brick convolution
  int64_t step = 0;
  std::map<std::tuple<int, int, int>, std::unique_ptr<Work>> work;
};

namespace {

int sync_weights(sfx_lnet net, cudaStream_t s) {
  for (int l = 0; l < NLAYERS; l++) {
    const Conv& c = net->layers[l];
    f32_to_bf16<<<nb(c.nw()), 256, 0, s>>>(net->P.p + c.off, net->W16[l].p, c.nw());
    flip(c.ci, c.co, net->W16[l].p, net->Wt16[l].p, s);
    pack(c.ci, c.co, net->W16[l].p, net->Wp16[l].p, s);
    pack(c.co, c.ci, net->Wt16[l].p, net->Wtp16[l].p, s);
  }
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

Grid3 coarse_of(Grid3 f) { return Grid3{(f.nx + 1) / 2, (f.ny + 1) / 2, (f.nz + 1) / 2}; }

int get_work(sfx_lnet net, int nx, int ny, int nz, int batch, Work** out) {
  for (int n : {nx, ny, nz})
    if (n < 9 || (n - 1) % 8 != 0) return fail(SFX_ERR_UNSUPPORTED, "node grid must have 8k+1 nodes per direction");
  if (batch < 1) return fail(SFX_ERR_INVALID, "batch must be positive");
  auto key = std::make_tuple(nx, ny, nz);
  auto it = net->work.find(key);
  if (it != net->work.end() && it->second->cap >= batch) {
    *out = it->second.get();
    return SFX_OK;
  }
  if (it != net->work.end()) {
    SFX_CUDA_TRY(cudaDeviceSynchronize());  // the old buffers may still be in use
    net->work.erase(it);
  }
  auto w = std::make_unique<Work>();
  w->cap = batch;
  const size_t B = size_t(batch);
  w->g[0] = Grid3{nx, ny, nz};
  for (int l = 1; l < 4; l++) w->g[l] = coarse_of(w->g[l - 1]);
  const size_t N0 = size_t(w->g[0].nodes()), N1 = size_t(w->g[1].nodes()), N2 = size_t(w->g[2].nodes()),
               N3 = size_t(w->g[3].nodes());
  std::vector<std::pair<DeviceBuf<bf16>*, size_t>> b16 = {
      {&w->X0, N0 * 16}, {&w->A0b, N0 * 16}, {&w->B0b, N0 * 16}, {&w->C1, N1 * 16},  {&w->A1b, N1 * 32},
      {&w->B1b, N1 * 32}, {&w->C2, N2 * 32}, {&w->A2b, N2 * 48}, {&w->B2b, N2 * 48}, {&w->C3, N3 * 48},
      {&w->A3b, N3 * 48}, {&w->D2b, N2 * 48}, {&w->E2, N2 * 32}, {&w->D1b, N1 * 32}, {&w->E1, N1 * 16},
      {&w->D0b, N0 * 16}, {&w->E0, N0 * 16}};
  bool ok = true;
  for (auto& e : b16) ok = ok && e.first->alloc(e.second * B) == cudaSuccess;
  ok = ok && w->D2.alloc(N2 * 48 * B) == cudaSuccess && w->D1.alloc(N1 * 32 * B) == cudaSuccess &&
       w->D0.alloc(N0 * 16 * B) == cudaSuccess && w->OUT.alloc(N0 * 16 * B) == cudaSuccess;
  const size_t big = std::max({N0 * 16, N1 * 32, N2 * 48}) * B;
  for (auto* b : {&w->gOUT, &w->gE0, &w->gD0, &w->gE1, &w->gD1, &w->gE2, &w->gD2, &w->gA3, &w->gC3, &w->gB2, &w->gA2,
                  &w->gC2, &w->gB1, &w->gA1, &w->gC1, &w->gB0, &w->gA0, &w->gpre, &w->tmpf})
    ok = ok && b->alloc(big) == cudaSuccess;
  ok = ok && w->gpre16.alloc(big) == cudaSuccess;
  size_t npart = 0;
  for (int l = 0; l < NLAYERS; l++)
    npart = std::max(npart, size_t(wgrad_blocks(w->g[kLevel[l]], batch)) * size_t(net->layers[l].nw()));
  ok = ok && w->part.alloc(npart) == cudaSuccess && w->red.alloc(size_t(48) * 27 * 48) == cudaSuccess &&
       w->err.alloc(N0 * B) == cudaSuccess;
  for (auto* b : {&w->ss, &w->scale, &w->tt, &w->inv_tt, &w->esum}) ok = ok && b->alloc(B) == cudaSuccess;
  ok = ok && w->seg.alloc(B * kSegChunks) == cudaSuccess;
  if (!ok) return fail(SFX_ERR_NOMEM, "network workspace allocation failed");
  *out = w.get();
  net->work[key] = std::move(w);
  return SFX_OK;
}

const float* bias_of(sfx_lnet net, int l) { return net->P.p + net->layers[l].off + net->layers[l].nw(); }

// per-sample residual scale: w->scale[b] = RMS of r_b
void input_scale(Work* w, int B, const float* r, cudaStream_t s) {
  const int64_t N = w->g[0].nodes();
  square<<<nb(int64_t(B) * 3 * N), 256, 0, s>>>(r, w->tmpf.p, int64_t(B) * 3 * N);
  segment_sums(w->tmpf.p, 3 * N, B, w->seg.p, w->ss.p, s);
  make_scale<<<1, 64, 0, s>>>(w->ss.p, 3 * N, B, w->scale.p);
}

int forward(sfx_lnet net, Work* w, int B, cudaStream_t s) {
  const Grid3* g = w->g;
  const int64_t N0 = g[0].nodes(), N1 = g[1].nodes(), N2 = g[2].nodes(), N3 = g[3].nodes();
  SFX_TRY(conv_fwd(16, 16, true, g[0], B, w->X0.p, net->Wp16[A0].p, bias_of(net, A0), w->A0b.p, nullptr, net->wait_error.dev, s));
  SFX_TRY(conv_fwd(16, 16, true, g[0], B, w->A0b.p, net->Wp16[B0L].p, bias_of(net, B0L), w->B0b.p, nullptr, net->wait_error.dev, s));
  sfx::nn::restrict_to<bf16, bf16><<<grid2(N1 * 16, B), 256, 0, s>>>(g[0], g[1], 16, w->B0b.p, w->C1.p, 0.125f);
  SFX_TRY(conv_fwd(16, 32, true, g[1], B, w->C1.p, net->Wp16[A1].p, bias_of(net, A1), w->A1b.p, nullptr, net->wait_error.dev, s));
  SFX_TRY(conv_fwd(32, 32, true, g[1], B, w->A1b.p, net->Wp16[B1L].p, bias_of(net, B1L), w->B1b.p, nullptr, net->wait_error.dev, s));
  sfx::nn::restrict_to<bf16, bf16><<<grid2(N2 * 32, B), 256, 0, s>>>(g[1], g[2], 32, w->B1b.p, w->C2.p, 0.125f);
  SFX_TRY(conv_fwd(32, 48, true, g[2], B, w->C2.p, net->Wp16[A2].p, bias_of(net, A2), w->A2b.p, nullptr, net->wait_error.dev, s));
  SFX_TRY(conv_fwd(48, 48, true, g[2], B, w->A2b.p, net->Wp16[B2L].p, bias_of(net, B2L), w->B2b.p, nullptr, net->wait_error.dev, s));
  sfx::nn::restrict_to<bf16, bf16><<<grid2(N3 * 48, B), 256, 0, s>>>(g[2], g[3], 48, w->B2b.p, w->C3.p, 0.125f);
  SFX_TRY(conv_fwd(48, 48, true, g[3], B, w->C3.p, net->Wp16[A3].p, bias_of(net, A3), w->A3b.p, nullptr, net->wait_error.dev, s));
  // D2 = P A3 + B2 ; E2 = relu(conv(D2))
  cudaMemsetAsync(w->D2.p, 0, sizeof(float) * N2 * 48 * B, s);
  sfx::nn::prolong_add<bf16><<<grid2(N2 * 48, B), 256, 0, s>>>(g[2], g[3], 48, w->A3b.p, w->D2.p, 1.f);
  add_bf16_into<<<nb(N2 * 48 * B), 256, 0, s>>>(w->B2b.p, w->D2.p, w->D2b.p, N2 * 48 * B);
  SFX_TRY(conv_fwd(48, 32, true, g[2], B, w->D2b.p, net->Wp16[U2].p, bias_of(net, U2), w->E2.p, nullptr, net->wait_error.dev, s));
  cudaMemsetAsync(w->D1.p, 0, sizeof(float) * N1 * 32 * B, s);
  sfx::nn::prolong_add<bf16><<<grid2(N1 * 32, B), 256, 0, s>>>(g[1], g[2], 32, w->E2.p, w->D1.p, 1.f);
  add_bf16_into<<<nb(N1 * 32 * B), 256, 0, s>>>(w->B1b.p, w->D1.p, w->D1b.p, N1 * 32 * B);
  SFX_TRY(conv_fwd(32, 16, true, g[1], B, w->D1b.p, net->Wp16[U1].p, bias_of(net, U1), w->E1.p, nullptr, net->wait_error.dev, s));
  cudaMemsetAsync(w->D0.p, 0, sizeof(float) * N0 * 16 * B, s);
  sfx::nn::prolong_add<bf16><<<grid2(N0 * 16, B), 256, 0, s>>>(g[0], g[1], 16, w->E1.p, w->D0.p, 1.f);
  add_bf16_into<<<nb(N0 * 16 * B), 256, 0, s>>>(w->B0b.p, w->D0.p, w->D0b.p, N0 * 16 * B);
  SFX_TRY(conv_fwd(16, 16, true, g[0], B, w->D0b.p, net->Wp16[U0].p, bias_of(net, U0), w->E0.p, nullptr, net->wait_error.dev, s));
  SFX_TRY(conv_fwd(16, 16, false, g[0], B, w->E0.p, net->Wp16[OUTL].p, bias_of(net, OUTL), nullptr, w->OUT.p, net->wait_error.dev, s));
  return SFX_OK;
}

// backward through one convolution: given the gradient of its output (post
// activation) gy, accumulate dW, db (summed over the batch) into G and write
// the input gradient to gx (fp32, overwritten) unless gx is null.
int conv_bwd(sfx_lnet net, Work* w, int l, Grid3 g, int B, const bf16* x, const bf16* y, const float* gy, float* gx,
              cudaStream_t s) {
  const Conv& c = net->layers[l];
  const int64_t rows = g.nodes() * B;
  act_bwd<<<nb(rows * c.co), 256, 0, s>>>(gy, y, c.relu, w->gpre.p, w->gpre16.p, rows * c.co);
  const int nch = wgrad_blocks(g, B);
  conv_wgrad(c.ci, c.co, g, B, x, w->gpre16.p, w->part.p, s);
  sfx::nn::reduce_chunks<<<nb(c.nw()), 256, 0, s>>>(w->part.p, nch, c.nw(), w->red.p);
  add_into<<<nb(c.nw()), 256, 0, s>>>(w->red.p, net->G.p + c.off, c.nw());
  bias_grad(c.co, w->gpre.p, rows, w->red.p, s);
  add_into<<<1, 64, 0, s>>>(w->red.p, net->G.p + c.off + c.nw(), c.co);
  if (gx) SFX_TRY(conv_fwd(c.co, c.ci, false, g, B, w->gpre16.p, net->Wtp16[l].p, nullptr, nullptr, gx, net->wait_error.dev, s));
  return SFX_OK;
}

int backward(sfx_lnet net, Work* w, int B, cudaStream_t s) {
  const Grid3* g = w->g;
  const int64_t N0 = g[0].nodes(), N1 = g[1].nodes(), N2 = g[2].nodes(), N3 = g[3].nodes();
  // output and up path
  SFX_TRY(conv_bwd(net, w, OUTL, g[0], B, w->E0.p, nullptr, w->gOUT.p, w->gE0.p, s));
  SFX_TRY(conv_bwd(net, w, U0, g[0], B, w->D0b.p, w->E0.p, w->gE0.p, w->gD0.p, s));
  cudaMemcpyAsync(w->gB0.p, w->gD0.p, sizeof(float) * N0 * 16 * B, cudaMemcpyDeviceToDevice, s);
  sfx::nn::restrict_to<float, float><<<grid2(N1 * 16, B), 256, 0, s>>>(g[0], g[1], 16, w->gD0.p, w->gE1.p, 1.f);
  SFX_TRY(conv_bwd(net, w, U1, g[1], B, w->D1b.p, w->E1.p, w->gE1.p, w->gD1.p, s));
  cudaMemcpyAsync(w->gB1.p, w->gD1.p, sizeof(float) * N1 * 32 * B, cudaMemcpyDeviceToDevice, s);
  sfx::nn::restrict_to<float, float><<<grid2(N2 * 32, B), 256, 0, s>>>(g[1], g[2], 32, w->gD1.p, w->gE2.p, 1.f);
  SFX_TRY(conv_bwd(net, w, U2, g[2], B, w->D2b.p, w->E2.p, w->gE2.p, w->gD2.p, s));
  cudaMemcpyAsync(w->gB2.p, w->gD2.p, sizeof(float) * N2 * 48 * B, cudaMemcpyDeviceToDevice, s);
  sfx::nn::restrict_to<float, float><<<grid2(N3 * 48, B), 256, 0, s>>>(g[2], g[3], 48, w->gD2.p, w->gA3.p, 1.f);
  // coarsest and down path
  SFX_TRY(conv_bwd(net, w, A3, g[3], B, w->C3.p, w->A3b.p, w->gA3.p, w->gC3.p, s));
  sfx::nn::prolong_add<float><<<grid2(N2 * 48, B), 256, 0, s>>>(g[2], g[3], 48, w->gC3.p, w->gB2.p, 0.125f);
  SFX_TRY(conv_bwd(net, w, B2L, g[2], B, w->A2b.p, w->B2b.p, w->gB2.p, w->gA2.p, s));
  SFX_TRY(conv_bwd(net, w, A2, g[2], B, w->C2.p, w->A2b.p, w->gA2.p, w->gC2.p, s));
  sfx::nn::prolong_add<float><<<grid2(N1 * 32, B), 256, 0, s>>>(g[1], g[2], 32, w->gC2.p, w->gB1.p, 0.125f);
  SFX_TRY(conv_bwd(net, w, B1L, g[1], B, w->A1b.p, w->B1b.p, w->gB1.p, w->gA1.p, s));
  SFX_TRY(conv_bwd(net, w, A1, g[1], B, w->C1.p, w->A1b.p, w->gA1.p, w->gC1.p, s));
  sfx::nn::prolong_add<float><<<grid2(N0 * 16, B), 256, 0, s>>>(g[0], g[1], 16, w->gC1.p, w->gB0.p, 0.125f);
  SFX_TRY(conv_bwd(net, w, B0L, g[0], B, w->A0b.p, w->B0b.p, w->gB0.p, w->gA0.p, s));
  SFX_TRY(conv_bwd(net, w, A0, g[0], B, w->X0.p, w->A0b.p, w->gA0.p, nullptr, s));
  return SFX_OK;
}

// a batch: forward, loss, backward (gradient summed over the samples into
// net->G); per-sample error sums land in w->esum and 1 / |t/s|^2 in w->inv_tt
int batch_grad(sfx_lnet net, Work* w, int B, const float* r, const float* t, const float* feat, cudaStream_t s) {
  const int64_t N = w->g[0].nodes();
  input_scale(w, B, r, s);
  pack_input<<<grid2(N, B), 256, 0, s>>>(r, feat, N, w->scale.p, w->X0.p);
  SFX_TRY(forward(net, w, B, s));
  target_sq<<<grid2(N, B), 256, 0, s>>>(t, feat, N, w->scale.p, w->tmpf.p);
  segment_sums(w->tmpf.p, N, B, w->seg.p, w->tt.p, s);
  make_inverse<<<1, 64, 0, s>>>(w->tt.p, B, w->inv_tt.p);
  loss_grad<<<grid2(N, B), 256, 0, s>>>(w->OUT.p, t, feat, N, w->scale.p, w->inv_tt.p, w->gOUT.p, w->err.p);
  segment_sums(w->err.p, N, B, w->seg.p, w->esum.p, s);
  SFX_TRY(backward(net, w, B, s));
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

// mean over the batch of esum[b] * inv_tt[b] (synchronises the stream)
int read_mean_loss(Work* w, int B, cudaStream_t s, float* loss) {
  std::vector<float> e(static_cast<size_t>(B)), itt(static_cast<size_t>(B));
  SFX_CUDA_TRY(cudaMemcpyAsync(e.data(), w->esum.p, sizeof(float) * B, cudaMemcpyDeviceToHost, s));
  SFX_CUDA_TRY(cudaMemcpyAsync(itt.data(), w->inv_tt.p, sizeof(float) * B, cudaMemcpyDeviceToHost, s));
  SFX_CUDA_TRY(cudaStreamSynchronize(s));
  double tot = 0.0;
  for (int b = 0; b < B; b++) tot += double(e[size_t(b)]) * itt[size_t(b)];
  *loss = float(tot / B);
  return SFX_OK;
}

}  // namespace

namespace sfx_impl {

int lnet_apply(sfx_lnet net, int nx, int ny, int nz, const float* r, const float* features, float* z,
               cudaStream_t s) {
  Work* w = nullptr;
  if (int rc = get_work(net, nx, ny, nz, 1, &w)) return rc;
  const int64_t N = w->g[0].nodes();
  input_scale(w, 1, r, s);
  pack_input<<<grid2(N, 1), 256, 0, s>>>(r, features, N, w->scale.p, w->X0.p);
  if (int rc = forward(net, w, 1, s)) return rc;
  unpack_output<<<grid2(N, 1), 256, 0, s>>>(w->OUT.p, features, N, w->scale.p, z);
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

// a convolution of an earlier (completed) call gave up a bounded wait
int check_waits(sfx_lnet net) {
  if (!net->wait_error.raised()) return SFX_OK;
  net->wait_error.clear();
  return fail(SFX_ERR_TIMEOUT, "a tensor-core wait of the network's convolution expired");
}

}  // namespace sfx_impl

extern "C" {

int sfx_lnet_create(uint64_t seed, sfx_lnet* out) {
  if (!out) return fail(SFX_ERR_INVALID, "null output");
  *out = nullptr;
  auto* net = new (std::nothrow) sfx_lnet_s;
  if (!net) return fail(SFX_ERR_NOMEM, "host allocation failed");
  const int spec[NLAYERS][3] = {{16, 16, 1}, {16, 16, 1}, {16, 32, 1}, {32, 32, 1}, {32, 48, 1}, {48, 48, 1},
                                {48, 48, 1}, {48, 32, 1}, {32, 16, 1}, {16, 16, 1}, {16, 16, 0}};
  int64_t off = 0;
  for (int l = 0; l < NLAYERS; l++) {
    net->layers[l] = Conv{spec[l][0], spec[l][1], spec[l][2] != 0, off};
    off += net->layers[l].nw() + spec[l][1];
  }
  net->nparams = off;
  std::vector<float> p(size_t(off), 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < NLAYERS; l++) {
    const Conv& c = net->layers[l];
    std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / (27.0 * c.ci)) * (c.relu ? 1.0 : 0.1));
    for (int64_t i = 0; i < c.nw(); i++) p[size_t(c.off + i)] = float(nd(rng));
  }
  bool ok = net->wait_error.init() == cudaSuccess && net->P.upload(p.data(), p.size()) == cudaSuccess &&
            net->G.alloc(p.size()) == cudaSuccess &&
            net->M.alloc(p.size()) == cudaSuccess && net->V.alloc(p.size()) == cudaSuccess;
  for (int l = 0; l < NLAYERS && ok; l++)
    ok = net->W16[l].alloc(size_t(net->layers[l].nw())) == cudaSuccess &&
         net->Wt16[l].alloc(size_t(net->layers[l].nw())) == cudaSuccess &&
         net->Wp16[l].alloc(size_t(net->layers[l].nw())) == cudaSuccess &&
         net->Wtp16[l].alloc(size_t(net->layers[l].nw())) == cudaSuccess;
  if (ok) ok = cudaMemset(net->M.p, 0, p.size() * 4) == cudaSuccess && cudaMemset(net->V.p, 0, p.size() * 4) == cudaSuccess;
  if (!ok || sync_weights(net, nullptr) != SFX_OK || cudaDeviceSynchronize() != cudaSuccess) {
    delete net;
    return fail(SFX_ERR_NOMEM, "network allocation failed");
  }
  *out = net;
  return SFX_OK;
}

int sfx_lnet_destroy(sfx_lnet net) {
  delete net;
  return SFX_OK;
}

int sfx_lnet_num_params(sfx_lnet net, int64_t* n) {
  if (!net || !n) return fail(SFX_ERR_INVALID, "null argument");
  *n = net->nparams;
  return SFX_OK;
}

int sfx_lnet_get_params(sfx_lnet net, float* host, int64_t n) {
  if (!net || !host || n != net->nparams) return fail(SFX_ERR_INVALID, "bad parameter buffer");
  SFX_CUDA_TRY(cudaMemcpy(host, net->P.p, sizeof(float) * size_t(n), cudaMemcpyDeviceToHost));
  return SFX_OK;
}

int sfx_lnet_set_params(sfx_lnet net, const float* host, int64_t n) {
  if (!net || !host || n != net->nparams) return fail(SFX_ERR_INVALID, "bad parameter buffer");
  SFX_CUDA_TRY(cudaMemcpy(net->P.p, host, sizeof(float) * size_t(n), cudaMemcpyHostToDevice));
  if (int rc = sync_weights(net, nullptr)) return rc;
  SFX_CUDA_TRY(cudaDeviceSynchronize());
  return SFX_OK;
}

int sfx_lnet_apply(sfx_lnet net, int nx, int ny, int nz, const float* r, const float* features, float* z,
                   void* stream) {
  if (!net || !r || !features || !z) return fail(SFX_ERR_INVALID, "null argument");
  if (int rc = check_waits(net)) return rc;
  return lnet_apply(net, nx, ny, nz, r, features, z, static_cast<cudaStream_t>(stream));
}

int sfx_lnet_gradient(sfx_lnet net, int nx, int ny, int nz, const float* r, const float* target,
                      const float* features, float* loss, float* grad_host, void* stream) {
  if (!net || !r || !target || !features || !loss || !grad_host) return fail(SFX_ERR_INVALID, "null argument");
  if (int rc = check_waits(net)) return rc;
  auto s = static_cast<cudaStream_t>(stream);
  Work* w = nullptr;
  if (int rc = get_work(net, nx, ny, nz, 1, &w)) return rc;
  SFX_CUDA_TRY(cudaMemsetAsync(net->G.p, 0, sizeof(float) * size_t(net->nparams), s));
  if (int rc = batch_grad(net, w, 1, r, target, features, s)) return rc;
  SFX_CUDA_TRY(cudaMemcpyAsync(grad_host, net->G.p, sizeof(float) * size_t(net->nparams), cudaMemcpyDeviceToHost, s));
  return read_mean_loss(w, 1, s, loss);
}

int sfx_lnet_train_step(sfx_lnet net, int nx, int ny, int nz, int batch, const float* r, const float* target,
                        const float* features, float lr, float* mean_loss, void* stream) {
  if (!net || !r || !target || !features || batch < 1) return fail(SFX_ERR_INVALID, "bad argument");
  if (int rc = check_waits(net)) return rc;
  auto s = static_cast<cudaStream_t>(stream);
  Work* w = nullptr;
  if (int rc = get_work(net, nx, ny, nz, batch, &w)) return rc;
  SFX_CUDA_TRY(cudaMemsetAsync(net->G.p, 0, sizeof(float) * size_t(net->nparams), s));
  if (int rc = batch_grad(net, w, batch, r, target, features, s)) return rc;
  net->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, float(net->step)), c2 = 1.f - std::pow(b2, float(net->step));
  adam<<<nb(net->nparams), 256, 0, s>>>(net->P.p, net->G.p, net->M.p, net->V.p, net->nparams, lr, b1, b2, c1, c2,
                                        1e-8f, 1.f / float(batch));
  if (int rc = sync_weights(net, s)) return rc;
  float l = 0.f;
  if (int rc = read_mean_loss(w, batch, s, &l)) return rc;
  if (mean_loss) *mean_loss = l;
  return check_waits(net);
}

}  // extern "C"
