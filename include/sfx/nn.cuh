// sfx — kernels of the learned multilevel preconditioner: 3x3x3 convolutions
// on node grids (channels-last BF16 activations, FP32 accumulation on the
// 5th-generation tensor cores through tcgen05.mma with tensor-memory
// accumulators for the forward and data-gradient convolutions, mma.sync
// m16n8k16 for the weight gradient), grid transfer between levels, and the
// backward passes used to train the network.
//
// A volume is an nx x ny x nz node grid with C channels (C a multiple of 16),
// stored [z][y][x][C].  Convolutions use zero padding, stride 1:
//   y[n][co] = act(b[co] + sum_{tap, ci} W[co][tap][ci] x[n + off(tap)][ci]),
// tap = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1).  Levels nest as 2m+1 -> m+1
// nodes per direction (the Q2 node grid of an n^3 mesh is (2n+1)^3).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "sfx/umma.cuh"

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

/// Brick of input nodes staged by conv3_fwd_brick: the 8 x 16 x BZ output
/// nodes of a block plus a one-node halo, (10 x 18 x (BZ + 2)) nodes, stored
/// as 2 * CIN / 16 slabs of 8 channels, each slab [z][y][x] x 16 bytes (what
/// one tiled TMA load of an 8-channel box writes).
template <int CIN, int BZ>
struct BrickLayout {
  static constexpr int BX = 8, BY = 16;
  static constexpr int XP = BX + 2, YP = BY + 2, ZP = BZ + 2;
  static constexpr int NODES = XP * YP * ZP;
  static constexpr int KC = CIN / 16;                      // 16-channel K-steps
  static constexpr uint32_t SLAB = uint32_t(NODES) * 16;    // bytes of one 8-channel slab
  static constexpr uint32_t BRICK = SLAB * 2 * KC;
};

/// output planes per block: 4 for the 16-channel inputs of the finest level,
/// 2 for the wider (coarser) layers, so the brick and the weights of all 27
/// taps fit in shared memory
__host__ __device__ constexpr int brick_bz(int cin) { return cin == 16 ? 4 : 2; }

template <int CIN, int COUT>
struct BrickConvSmem {
  static constexpr int BZ = brick_bz(CIN);
  using Brick = BrickLayout<CIN, BZ>;
  static constexpr uint32_t W_BYTES = 27u * COUT * CIN * 2;  // all taps, [tap][kc][half][co] x 16 bytes
  static constexpr size_t bytes = size_t(Brick::BRICK) + W_BYTES;
  static constexpr uint32_t cols = uint32_t(BZ) * COUT;       // BZ accumulators of COUT FP32 columns
  static constexpr uint32_t NCOLS = cols <= 32 ? 32 : cols <= 64 ? 64 : cols <= 128 ? 128 : 256;
};

/// The weights W[co][tap][ci] of a brick convolution in its shared-memory
/// order, [tap][ci / 8][co] x 8 BF16 (K-major core matrices per tap and
/// K-step), so that one bulk copy stages all 27 taps.  One thread per
/// 16-byte group of W.
template <int CIN, int COUT>
__global__ void pack_brick_weights(const __nv_bfloat16* __restrict__ W, __nv_bfloat16* __restrict__ Wp) {
  constexpr int GPN = CIN / 8;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= COUT * 27 * GPN) return;
  const int g8 = i % GPN, tap = (i / GPN) % 27, co = i / (GPN * 27);
  reinterpret_cast<uint4*>(Wp)[(tap * GPN + g8) * COUT + co] = reinterpret_cast<const uint4*>(W)[i];
}

/// Forward 3x3x3 convolution as an implicit GEMM on the 5th-generation tensor
/// cores with a shared-memory brick: each block owns 8 x 16 x BZ output nodes
/// of one sample.  One thread loads the brick with its halo by tiled TMA
/// (2 CIN / 16 loads of an 8-channel box through the tensor map `xmap` of the
/// activations [sample][z][y][x][CIN]; halo nodes outside the grid read
/// zero) and the weights of all 27 taps, pre-packed as K-major core matrices
/// (pack_brick_weights), by one bulk copy, all on one mbarrier.  For a tap (dx, dy, dz) the A operand of output plane zt (128
/// rows = 8 x by 16 y nodes) is then the brick itself read through a shifted
/// descriptor: row group y starts at node ((zt + dz + 1) 18 + y + dy + 1) 10 +
/// dx + 1 (leading byte offset = one slab between channel halves, stride
/// byte offset = one brick row of 10 nodes between row groups), so no tap
/// is ever gathered.  One thread issues the 27 x BZ x CIN / 16 MMAs into BZ
/// tensor-memory accumulators and commits them; the epilogue reads them with
/// tcgen05.ld (warp w: rows 32w..32w+31 of each plane), adds the bias,
/// applies the activation and stores BF16 (or FP32 into y_f32).  Wp: the
/// packed weights (27 COUT CIN bf16, 16-byte aligned), bias: [COUT] f32 (may
/// be null), y: [node][COUT] per sample.
/// Every wait is bounded: on a timeout the block sets *err, waits (bounded)
/// for its copies and MMAs in flight and frees its tensor memory.
template <int CIN, int COUT, int ACT>
__global__ void __launch_bounds__(128, 1) conv3_fwd_brick(const __grid_constant__ CUtensorMap xmap, Grid3 g,
                                                       const __nv_bfloat16* __restrict__ Wp,
                                                       const float* __restrict__ bias, __nv_bfloat16* __restrict__ y,
                                                       float* __restrict__ y_f32, int* __restrict__ err) {
  static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 64, "channel counts");
  using L = BrickConvSmem<CIN, COUT>;
  using Bk = typename L::Brick;
  constexpr int BZ = L::BZ;
  extern __shared__ __align__(128) unsigned char sfx_conv_smem[];
  __shared__ uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_base;
  unsigned char* brick = sfx_conv_smem;
  unsigned char* wsm = sfx_conv_smem + Bk::BRICK;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nbx = (g.nx + Bk::BX - 1) / Bk::BX, nby = (g.ny + Bk::BY - 1) / Bk::BY;
  const int bx = int(blockIdx.x % unsigned(nbx)), by = int((blockIdx.x / unsigned(nbx)) % unsigned(nby));
  const int bz = int(blockIdx.x / unsigned(nbx * nby));
  const int sample = int(blockIdx.y);
  const int64_t N = g.nodes();
  if (threadIdx.x == 0) {
    bulk::mbar_init(&bar_load, 1);
    bulk::mbar_init(&bar_mma, 1);
    bulk::fence_mbar_init();
  }
  if (warp == 0) {
    umma::tmem_alloc(&tmem_base, L::NCOLS);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;
  constexpr int GPN = CIN / 8;
  if (threadIdx.x == 0) {
    bulk::mbar_arrive_expect_tx(&bar_load, Bk::BRICK + L::W_BYTES);
#pragma unroll
    for (int sl = 0; sl < 2 * Bk::KC; sl++)
      bulk::tma_load_5d(brick + uint32_t(sl) * Bk::SLAB, &xmap, sl * 8, bx * Bk::BX - 1, by * Bk::BY - 1, bz * BZ - 1,
                        sample, &bar_load);
    bulk::copy_g2s(wsm, Wp, L::W_BYTES, &bar_load);
  }
  bool ok = __syncthreads_and(bulk::mbar_wait(&bar_load, 0u));
  umma::fence_after_sync();
  if (ok && threadIdx.x == 0) {
    constexpr uint32_t idesc = umma::idesc_bf16_f32(128, COUT);
    for (int tap = 0; tap < 27; tap++) {
      const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
#pragma unroll
      for (int zt = 0; zt < BZ; zt++) {
        const uint32_t n0 = uint32_t(((zt + dz + 1) * Bk::YP + (dy + 1)) * Bk::XP + (dx + 1));
#pragma unroll
        for (int kc = 0; kc < Bk::KC; kc++) {
          const uint64_t adesc = umma::smem_desc(brick + uint32_t(2 * kc) * Bk::SLAB + n0 * 16u, Bk::SLAB, Bk::XP * 16);
          const uint64_t bdesc = umma::smem_desc(wsm + (uint32_t(tap) * GPN + 2 * kc) * COUT * 16u, COUT * 16, 128);
          umma::mma_bf16(tmem + uint32_t(zt * COUT), adesc, bdesc, idesc, tap > 0 || kc > 0);
        }
      }
    }
    umma::commit(&bar_mma);
  }
  const bool issued = ok;
  if (ok) ok = __syncthreads_and(bulk::mbar_wait(&bar_mma, 0u));
  umma::fence_after_sync();
  if (ok) {
    const int r = 32 * warp + lane;  // row of every plane's tile: 8 x by 16 y
    const int ox = bx * Bk::BX + (r & 7), oy = by * Bk::BY + (r >> 3);
#pragma unroll
    for (int zt = 0; zt < BZ; zt++) {
      const int oz = bz * BZ + zt;
      const bool inside = ox < g.nx && oy < g.ny && oz < g.nz;
      const int64_t n = int64_t(sample) * N + (int64_t(oz) * g.ny + oy) * g.nx + ox;
#pragma unroll
      for (int c = 0; c < COUT; c += 8) {
        float v[8];
        umma::ld_x8(tmem + (uint32_t(32 * warp) << 16) + uint32_t(zt * COUT + c), v);
        if (inside) {
#pragma unroll
          for (int i = 0; i < 8; i++) {
            float t = v[i] + (bias ? bias[c + i] : 0.f);
            if (ACT == ACT_RELU) t = t > 0.f ? t : 0.f;
            v[i] = t;
          }
          if (y_f32) {
#pragma unroll
            for (int i = 0; i < 8; i++) y_f32[n * COUT + c + i] = v[i];
          } else {
            const uint4 pk = make_uint4(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]), pack_bf16x2(v[4], v[5]),
                                        pack_bf16x2(v[6], v[7]));
            *reinterpret_cast<uint4*>(y + n * COUT + c) = pk;
          }
        }
      }
    }
  } else {
    if (threadIdx.x == 0) atomicExch(err, 1);
    // the copies and MMAs in flight (bounded) before the tensor memory is released
    (void)bulk::mbar_wait(&bar_load, 0u);
    if (issued) (void)bulk::mbar_wait(&bar_mma, 0u);
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::tmem_dealloc(tmem, L::NCOLS);
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
