// sfx — kernels of the learned multilevel preconditioner: 3x3x3 convolutions
// on node grids (channels-last BF16 activations, FP32 accumulation on the
// tensor cores through mma.sync m16n8k16), grid transfer between levels, and
// the backward passes used to train the network.
//
// A volume is an nx x ny x nz node grid with C channels (C a multiple of 16),
// stored [z][y][x][C].  Convolutions use zero padding, stride 1:
//   y[n][co] = act(b[co] + sum_{tap, ci} W[co][tap][ci] x[n + off(tap)][ci]),
// tap = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1).  Levels nest as 2m+1 -> m+1
// nodes per direction (the Q2 node grid of an n^3 mesh is (2n+1)^3).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace sfx {
namespace nn {

struct Grid3 {
  int nx, ny, nz;
  __host__ __device__ int64_t nodes() const { return int64_t(nx) * ny * nz; }
};

__device__ inline uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ inline void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

enum Act : int { ACT_NONE = 0, ACT_RELU = 1 };

/// Shared-memory layout of conv3_fwd for CIN input and COUT output channels:
/// the input rows of the block's 64 output nodes for each of the 9 (dy, dz)
/// neighbour offsets (66 consecutive nodes each, a row stride of CIN + 8 bf16)
/// and the whole weight tensor (per output channel 27 * CIN + 8 bf16).  The
/// padding makes the mma fragment loads of 8 rows x 4 lanes hit 32 banks.
template <int CIN, int COUT>
struct ConvSmem {
  static constexpr int NODES = 64;         // output nodes per block (4 warps x 16)
  static constexpr int SEG = NODES + 2;    // staged source nodes per (dy, dz) offset
  static constexpr int RS = CIN + 8;       // input row stride (bf16)
  static constexpr int WS = 27 * CIN + 8;  // weight row stride per output channel (bf16)
  static constexpr size_t x_elems = size_t(9) * SEG * RS;
  static constexpr size_t w_elems = size_t(COUT) * WS;
  static constexpr size_t bytes = (x_elems + w_elems) * 2;
};

/// Forward 3x3x3 convolution as an implicit GEMM on mma.sync m16n8k16 (BF16 in,
/// FP32 accumulate).  A block of 4 warps computes 64 consecutive output nodes
/// (16 per warp) for all COUT channels; the input rows they touch and the
/// weights are first staged in shared memory (16-byte vector loads), then the
/// K loop runs over the 27 taps and the input channels in chunks of 16.
/// x: [node][CIN] bf16, W: [COUT][27][CIN] bf16, bias: [COUT] f32 (may be
/// null), y: [node][COUT] bf16.  If `y_f32` is non-null the pre-cast FP32
/// result is written there instead.  blockIdx.y selects the sample of a batch
/// (volumes stored one after another).  Dynamic shared memory:
/// ConvSmem<CIN, COUT>::bytes.
template <int CIN, int COUT, int ACT>
__global__ void __launch_bounds__(128) conv3_fwd(Grid3 g, const __nv_bfloat16* __restrict__ x,
                                                 const __nv_bfloat16* __restrict__ W, const float* __restrict__ bias,
                                                 __nv_bfloat16* __restrict__ y, float* __restrict__ y_f32) {
  static_assert(CIN % 16 == 0 && COUT % 8 == 0, "channel counts");
  using L = ConvSmem<CIN, COUT>;
  constexpr int NT = COUT / 8;
  extern __shared__ __align__(16) unsigned char sfx_conv_smem[];
  __nv_bfloat16* sx = reinterpret_cast<__nv_bfloat16*>(sfx_conv_smem);
  __nv_bfloat16* sw = sx + L::x_elems;
  const int64_t N = g.nodes();
  const int64_t n0 = int64_t(blockIdx.x) * L::NODES;
  x += int64_t(blockIdx.y) * N * CIN;
  if (y) y += int64_t(blockIdx.y) * N * COUT;
  if (y_f32) y_f32 += int64_t(blockIdx.y) * N * COUT;

  // stage the weights: W[co][tap][ci] -> sw[co * WS + tap * CIN + ci]
  {
    constexpr int VPR = 27 * CIN / 8;  // 16-byte vectors per output channel
    const uint4* src = reinterpret_cast<const uint4*>(W);
    for (int i = threadIdx.x; i < COUT * VPR; i += blockDim.x) {
      const int co = i / VPR, v = i % VPR;
      *reinterpret_cast<uint4*>(sw + co * L::WS + v * 8) = src[i];
    }
  }
  // stage the input rows: segment k = (dz + 1) * 3 + (dy + 1) holds nodes
  // n0 - 1 + dy nx + dz nx ny + [0, SEG) (zeros outside [0, N))
  {
    constexpr int VPN = CIN / 8;  // 16-byte vectors per node
    const uint4* src = reinterpret_cast<const uint4*>(x);
    const int64_t plane = int64_t(g.nx) * g.ny;
    for (int i = threadIdx.x; i < 9 * L::SEG * VPN; i += blockDim.x) {
      const int k = i / (L::SEG * VPN), rem = i % (L::SEG * VPN);
      const int j = rem / VPN, v = rem % VPN;
      const int dy = k % 3 - 1, dz = k / 3 - 1;
      const int64_t node = n0 - 1 + dy * int64_t(g.nx) + dz * plane + j;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (node >= 0 && node < N) val = src[node * VPN + v];
      *reinterpret_cast<uint4*>(sx + (size_t(k) * L::SEG + j) * L::RS + v * 8) = val;
    }
  }
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  // the two rows (output nodes) this lane feeds into the A fragment
  int ln[2] = {warp * 16 + gid, warp * 16 + gid + 8};  // local index in [0, 64)
  int rx[2], ry[2], rz[2];
  bool rv[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int64_t n = n0 + ln[h];
    rv[h] = n < N;
    const int64_t nn = rv[h] ? n : 0;
    rx[h] = int(nn % g.nx);
    ry[h] = int((nn / g.nx) % g.ny);
    rz[h] = int(nn / (int64_t(g.nx) * g.ny));
  }
  float acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; j++)
#pragma unroll
    for (int k = 0; k < 4; k++) acc[j][k] = 0.f;

#pragma unroll 1
  for (int tap = 0; tap < 27; tap++) {
    const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
    const int seg = (dz + 1) * 3 + (dy + 1);
    const __nv_bfloat16* rowp[2];
    bool sv[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int xx = rx[h] + dx, yy = ry[h] + dy, zz = rz[h] + dz;
      sv[h] = rv[h] && xx >= 0 && xx < g.nx && yy >= 0 && yy < g.ny && zz >= 0 && zz < g.nz;
      rowp[h] = sx + (size_t(seg) * L::SEG + (ln[h] + 1 + dx)) * L::RS;
    }
#pragma unroll
    for (int kc = 0; kc < CIN / 16; kc++) {
      const int c0 = kc * 16 + tig * 2;
      uint32_t a[4];
      a[0] = sv[0] ? *reinterpret_cast<const uint32_t*>(rowp[0] + c0) : 0u;
      a[1] = sv[1] ? *reinterpret_cast<const uint32_t*>(rowp[1] + c0) : 0u;
      a[2] = sv[0] ? *reinterpret_cast<const uint32_t*>(rowp[0] + c0 + 8) : 0u;
      a[3] = sv[1] ? *reinterpret_cast<const uint32_t*>(rowp[1] + c0 + 8) : 0u;
#pragma unroll
      for (int j = 0; j < NT; j++) {
        const __nv_bfloat16* wr = sw + (j * 8 + gid) * L::WS + tap * CIN + c0;
        uint32_t b[2] = {*reinterpret_cast<const uint32_t*>(wr), *reinterpret_cast<const uint32_t*>(wr + 8)};
        mma_bf16_16816(acc[j], a, b);
      }
    }
  }
  // epilogue: rows gid / gid+8, columns j*8 + tig*2 + {0,1}
#pragma unroll
  for (int j = 0; j < NT; j++) {
    const int co = j * 8 + tig * 2;
    const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      if (!rv[h]) continue;
      const int64_t n = n0 + ln[h];
      float v0 = acc[j][2 * h] + b0, v1 = acc[j][2 * h + 1] + b1;
      if (ACT == ACT_RELU) {
        v0 = v0 > 0.f ? v0 : 0.f;
        v1 = v1 > 0.f ? v1 : 0.f;
      }
      if (y_f32) {
        y_f32[n * COUT + co] = v0;
        y_f32[n * COUT + co + 1] = v1;
      } else {
        reinterpret_cast<uint32_t*>(y)[(n * COUT + co) >> 1] = pack_bf16x2(v0, v1);
      }
    }
  }
}

/// Weights of the data-gradient convolution: Wt[ci][tap][co] = W[co][26 - tap][ci].
template <int CIN, int COUT>
__global__ void flip_weights(const __nv_bfloat16* __restrict__ W, __nv_bfloat16* __restrict__ Wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= CIN * 27 * COUT) return;
  const int co = i % COUT, tap = (i / COUT) % 27, ci = i / (COUT * 27);
  Wt[(int64_t(ci) * 27 + tap) * COUT + co] = W[(int64_t(co) * 27 + (26 - tap)) * CIN + ci];
}

/// Weight gradient on the tensor cores:
///   dW[co][tap][ci] = sum_n dy[n][co] x[n + off(tap)][ci]
/// as a GEMM with M = COUT, N = CIN per tap and K = nodes of all samples of
/// the batch.  Each sample's nodes are cut into chunks of kWgradChunk; block b
/// takes chunks b, b + gridDim.x, ... of the batch's chunk list and
/// writes its partial sums to part[b][co][tap][ci] (reduced over blocks in
/// fixed order by reduce_chunks).  Per chunk the block stages dy^T
/// ([co][node], BF16) and the tap-shifted x^T ([ci][node], zero outside the
/// grid) in shared memory; its four warps take interleaved 16-node k-steps
/// and are summed in warp order at the end of each tap.
constexpr int kWgradChunk = 128;

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) conv3_wgrad_mma(Grid3 g, int batch, const __nv_bfloat16* __restrict__ x,
                                                       const __nv_bfloat16* __restrict__ dy, float* __restrict__ part) {
  static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channel counts");
  constexpr int KC = kWgradChunk;
  constexpr int LD = KC + 8;  // row pitch in BF16: 68 words, 4 mod 32 -> conflict-free fragment loads
  constexpr int MT = COUT / 16, NT = CIN / 8, T = MT * NT;
  __shared__ __align__(16) __nv_bfloat16 sA[COUT * LD];
  __shared__ __align__(16) __nv_bfloat16 sB[CIN * LD];
  __shared__ float sR[T * 4 * 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int64_t N = g.nodes();
  const int64_t per_sample = (N + KC - 1) / KC;
  const int64_t nchunks = per_sample * batch;
  const bool one_chunk = int64_t(blockIdx.x) + gridDim.x >= nchunks;  // dy^T staged once for all taps
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
#pragma unroll 1
  for (int tap = 0; tap < 27; tap++) {
    const int ox = tap % 3 - 1, oy = (tap / 3) % 3 - 1, oz = tap / 9 - 1;
    float acc[T][4];
#pragma unroll
    for (int t = 0; t < T; t++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[t][j] = 0.f;
#pragma unroll 1
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
      const int64_t smp = c / per_sample;
      const int64_t b0 = (c - smp * per_sample) * KC;
      const __nv_bfloat16* xs = x + smp * N * CIN;
      const __nv_bfloat16* dys = dy + smp * N * COUT;
      __syncthreads();  // the previous k-steps are done with sA / sB
      if (!one_chunk || tap == 0) {
        for (int i = threadIdx.x; i < KC * COUT; i += blockDim.x) {
          const int k = i / COUT, co = i % COUT;
          const int64_t n = b0 + k;
          sA[co * LD + k] = n < N ? dys[n * COUT + co] : zero;
        }
      }
      for (int i = threadIdx.x; i < KC * CIN; i += blockDim.x) {
        const int k = i / CIN, ci = i % CIN;
        const int64_t n = b0 + k;
        __nv_bfloat16 v = zero;
        if (n < N) {
          const int xx = int(n % g.nx) + ox, yy = int((n / g.nx) % g.ny) + oy,
                    zz = int(n / (int64_t(g.nx) * g.ny)) + oz;
          if (xx >= 0 && xx < g.nx && yy >= 0 && yy < g.ny && zz >= 0 && zz < g.nz)
            v = xs[((int64_t(zz) * g.ny + yy) * g.nx + xx) * CIN + ci];
        }
        sB[ci * LD + k] = v;
      }
      __syncthreads();
#pragma unroll 1
      for (int ks = warp; ks < KC / 16; ks += 4) {
        const int k0 = ks * 16 + tig * 2;
        uint32_t a[MT][4];
#pragma unroll
        for (int mt = 0; mt < MT; mt++) {
          const __nv_bfloat16* r0 = sA + (mt * 16 + gid) * LD + k0;
          const __nv_bfloat16* r1 = r0 + 8 * LD;
          a[mt][0] = *reinterpret_cast<const uint32_t*>(r0);
          a[mt][1] = *reinterpret_cast<const uint32_t*>(r1);
          a[mt][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
          a[mt][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        }
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
          const __nv_bfloat16* rb = sB + (nt * 8 + gid) * LD + k0;
          const uint32_t b[2] = {*reinterpret_cast<const uint32_t*>(rb), *reinterpret_cast<const uint32_t*>(rb + 8)};
#pragma unroll
          for (int mt = 0; mt < MT; mt++) mma_bf16_16816(acc[mt * NT + nt], a[mt], b);
        }
      }
    }
    // sum the four warps' tiles in warp order, then store this tap's partials
#pragma unroll 1
    for (int w = 0; w < 4; w++) {
      if (warp == w) {
#pragma unroll
        for (int t = 0; t < T; t++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            float* r = &sR[(t * 4 + j) * 32 + lane];
            *r = (w == 0 ? 0.f : *r) + acc[t][j];
          }
      }
      __syncthreads();
    }
    float* out = part + int64_t(blockIdx.x) * COUT * 27 * CIN;
    for (int i = threadIdx.x; i < T * 128; i += blockDim.x) {
      const int t = i >> 7, j = (i >> 5) & 3, l = i & 31;
      const int mt = t / NT, nt = t % NT;
      const int co = mt * 16 + (l >> 2) + (j >= 2 ? 8 : 0);
      const int ci = nt * 8 + (l & 3) * 2 + (j & 1);
      out[(int64_t(co) * 27 + tap) * CIN + ci] = sR[i];
    }
    __syncthreads();  // sR is rewritten by the next tap
  }
}

/// out[i] = sum_b part[b][i] (fixed order), optionally into a bias gradient too.
__global__ void reduce_chunks(const float* __restrict__ part, int nchunks, int64_t len, float* __restrict__ out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= len) return;
  float acc = 0.f;
  for (int b = 0; b < nchunks; b++) acc += part[int64_t(b) * len + i];
  out[i] = acc;
}

/// bias gradient db[co] = sum_n dy[n][co] (one block per channel, fixed-order tree)
template <int COUT>
__global__ void __launch_bounds__(256) bias_grad(const float* __restrict__ dy, int64_t N, float* __restrict__ db) {
  __shared__ float sh[256];
  const int co = blockIdx.x;
  float acc = 0.f;
  for (int64_t n = threadIdx.x; n < N; n += 256) acc += dy[n * COUT + co];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[co] = sh[0];
}

template <typename T>
__device__ inline float to_f(T v) {
  return float(v);
}
template <>
__device__ inline float to_f<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

/// Prolongation from the (m+1)-grid to the (2m+1)-grid by trilinear
/// interpolation (per channel), added into fine: fine += scale * P coarse.
/// blockIdx.y selects the sample.
template <typename T>
__global__ void prolong_add(Grid3 fg, Grid3 cg, int C, const T* __restrict__ coarse, float* __restrict__ fine,
                            float scale) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= fg.nodes() * C) return;
  coarse += int64_t(blockIdx.y) * cg.nodes() * C;
  fine += int64_t(blockIdx.y) * fg.nodes() * C;
  const int c = int(i % C);
  const int64_t n = i / C;
  const int x = int(n % fg.nx), y = int((n / fg.nx) % fg.ny), z = int(n / (int64_t(fg.nx) * fg.ny));
  const int x0 = x >> 1, y0 = y >> 1, z0 = z >> 1;
  const int x1 = x0 + (x & 1), y1 = y0 + (y & 1), z1 = z0 + (z & 1);
  float v = 0.f;
  const int xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int d = 0; d < 2; d++) {
        const int64_t cn = (int64_t(zs[a]) * cg.ny + ys[b]) * cg.nx + xs[d];
        v += 0.125f * to_f(coarse[cn * C + c]);
      }
  fine[i] += scale * v;
}

/// Restriction coarse = scale * P^T fine (scale 1/8: full weighting), any
/// input type; blockIdx.y selects the sample.
template <typename T, typename U>
__global__ void restrict_to(Grid3 fg, Grid3 cg, int C, const T* __restrict__ fine, U* __restrict__ coarse,
                            float scale) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= cg.nodes() * C) return;
  fine += int64_t(blockIdx.y) * fg.nodes() * C;
  coarse += int64_t(blockIdx.y) * cg.nodes() * C;
  const int c = int(i % C);
  const int64_t n = i / C;
  const int X = int(n % cg.nx), Y = int((n / cg.nx) % cg.ny), Z = int(n / (int64_t(cg.nx) * cg.ny));
  float v = 0.f;
  for (int dz = -1; dz <= 1; dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        const int x = 2 * X + dx, y = 2 * Y + dy, z = 2 * Z + dz;
        if (x < 0 || x >= fg.nx || y < 0 || y >= fg.ny || z < 0 || z >= fg.nz) continue;
        const float w = (dx ? 0.5f : 1.f) * (dy ? 0.5f : 1.f) * (dz ? 0.5f : 1.f);
        v += w * to_f(fine[((int64_t(z) * fg.ny + y) * fg.nx + x) * C + c]);
      }
  coarse[i] = U(scale * v);
}

}  // namespace nn
}  // namespace sfx
