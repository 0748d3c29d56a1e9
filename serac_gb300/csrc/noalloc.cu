// Residual of a structured hexahedral mesh that allocates nothing.
//
// For callers that cannot allocate device memory at all (for example code
// running under a memory manager that owns every device allocation, or code
// that must not grow the device footprint after start-up): the caller passes
// the vertex coordinates, the field and the output vector, connectivity and
// geometry are derived from the structured grid inside the kernels, and the
// element-residual scratch lives in a fixed file-scope device array.
//
// The array is per device, shared by every call on that device, and keeps the
// previous call's contents (every entry a call reads it writes first, so
// nothing needs clearing).  Calls that overlap on the GPU (different streams,
// or different host threads, on the same device) race on it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "form.hpp"
#include "sfx.h"
#include "sfx/kernels.cuh"
#include "sfx/materials.hpp"

namespace {

// 32 MiB of element-residual scratch: num_elements * components * (order+1)^3 doubles
constexpr int64_t kScratchDoubles = int64_t(4) * 1024 * 1024;
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_ptr[kMaxDevices] = {};
void* g_scratch_ctx[kMaxDevices] = {};  // the context each cached address belongs to

// The driver's current context (cuCtxGetCurrent, reached through the runtime
// so the library needs no link against the driver library).  A device reset
// or a new primary context reloads the module, and the array may then sit at
// another address: the cache is keyed by the context as well as the device.
int current_context(void** ctx) {
  using GetCtx = int (*)(void**);
  static GetCtx fn = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<GetCtx>(p);
    looked_up = true;
  }
  *ctx = nullptr;
  if (!fn || fn(ctx) != 0) return sfx_impl::fail(SFX_ERR_CUDA, "cuCtxGetCurrent failed");
  return SFX_OK;
}

// Device address of the scratch array for the current device and context
// (looked up once per device and context; the host-side symbol is only a
// stand-in for it and is never handed to a kernel).
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return sfx_impl::fail(SFX_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(err));
  if (dev < 0 || dev >= kMaxDevices) return sfx_impl::fail(SFX_ERR_UNSUPPORTED, "device index out of range");
  // (before the runtime's first use of the device the context is still null:
  // the lookup below creates it, and the next call caches its real handle)
  void* ctx = nullptr;
  if (int rc = current_context(&ctx)) return rc;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess)
      return sfx_impl::fail(SFX_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(err));
    g_scratch_ptr[dev] = static_cast<double*>(p);
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return SFX_OK;
}

struct Grid {
  int nx, ny, nz, p;
  int64_t Nx, Ny, Nz;
};

// element-local node a of element e -> global node
__device__ inline int64_t grid_node(const Grid& g, int64_t e, int kx, int ky, int kz) {
  int64_t ex = e % g.nx, ey = (e / g.nx) % g.ny, ez = e / (int64_t(g.nx) * g.ny);
  return (g.p * ex + kx) + g.Nx * ((g.p * ey + ky) + g.Ny * (g.p * ez + kz));
}

template <int P, int C, typename State, typename QF>
__global__ void __launch_bounds__(128) structured_residual_kernel(Grid g, QF qf, const double* __restrict__ vertices,
                                                                  const double* __restrict__ u, double* __restrict__ E,
                                                                  double t) {
  using namespace sfx;
  using namespace sfx::kernels;
  using Real = double;
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q * Q;
  constexpr int EPW = 32 / NQ;
  const int64_t ne = int64_t(g.nx) * g.ny * g.nz;
  const int64_t nn = g.Nx * g.Ny * g.Nz;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / NQ;
  const int qi_raw = lane - sub * NQ;
  const bool slot = sub < EPW;
  const int qi = slot ? qi_raw : NQ - 1;
  const int base = slot ? sub * NQ : 0;
  const int64_t e = warp * EPW + (slot ? sub : 0);
  const bool valid = slot && e < ne;
  const int ix = qi % Q, iy = (qi / Q) % Q, iz = qi / (Q * Q);

  __shared__ Real sB[Q][Q], sG[Q][Q];
  if (threadIdx.x < Q * Q) {
    int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = basis_table<P>().B[i][j];
    sG[i][j] = basis_table<P>().G[i][j];
  }
  __syncthreads();

  // geometry of this lane's point from the 8 vertices (trilinear map)
  tensor<Real, 3> X{};
  tensor<Real, 3, 3> Jm{};
  Real dvol = 0;
  tensor<Real, 3, 3> Ji = Identity<3>();
  if (valid) {
    const int64_t ex = e % g.nx, ey = (e / g.nx) % g.ny, ez = e / (int64_t(g.nx) * g.ny);
    const double s[3] = {gl_point(Q, ix), gl_point(Q, iy), gl_point(Q, iz)};
    for (int v = 0; v < 8; v++) {
      const int b0 = v & 1, b1 = (v >> 1) & 1, b2 = (v >> 2) & 1;
      const int64_t vid = (ex + b0) + int64_t(g.nx + 1) * ((ey + b1) + int64_t(g.ny + 1) * (ez + b2));
      const double N0 = b0 ? s[0] : 1.0 - s[0], N1 = b1 ? s[1] : 1.0 - s[1], N2 = b2 ? s[2] : 1.0 - s[2];
      const double d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0, d2 = b2 ? 1.0 : -1.0;
      const double phi = N0 * N1 * N2;
      const double gr[3] = {d0 * N1 * N2, N0 * d1 * N2, N0 * N1 * d2};
      for (int i = 0; i < 3; i++) {
        const double xv = vertices[vid * 3 + i];
        X[i] += xv * phi;
        for (int j = 0; j < 3; j++) Jm[i][j] += xv * gr[j];
      }
    }
    Ji = inv(Jm);
    dvol = det(Jm) * (gl_weight(Q, ix) * gl_weight(Q, iy) * gl_weight(Q, iz));
  }
  const int64_t node = valid ? grid_node(g, e, ix, iy, iz) : 0;

  value_t<C, Real> uv{};
  grad_t<C, Real> ug{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? u[c * nn + node] : Real(0);
    Real gg[3];
    interpolate_lane<Q, Real>(U, base, ix, iy, iz, sB, sG, comp<C>(uv, c), gg[0], gg[1], gg[2]);
#pragma unroll
    for (int j = 0; j < 3; j++) comp<C>(ug, c)[j] = gg[0] * Ji[0][j] + gg[1] * Ji[1][j] + gg[2] * Ji[2][j];
  }
  State st{};
  auto out = invoke_qf<State>(qf, t, tuple{X, Jm}, st, tuple{uv, ug});
  using SrcT = std::decay_t<decltype(get<0>(out))>;
  using FluxT = std::decay_t<decltype(get<1>(out))>;
  constexpr bool HS = has_part<RESIDUAL, SrcT>();
  constexpr bool HF = has_part<RESIDUAL, FluxT>();
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real sv = 0, f[3] = {0, 0, 0};
    if constexpr (HS) sv = dvol * part<RESIDUAL, Real>(source_comp<C>(get<0>(out), c));
    if constexpr (HF) {
      auto frow = flux_row<C>(get<1>(out), c);
      Real fp[3];
#pragma unroll
      for (int m = 0; m < 3; m++) fp[m] = part<RESIDUAL, Real>(frow[m]);
#pragma unroll
      for (int k = 0; k < 3; k++) f[k] = dvol * (fp[0] * Ji[k][0] + fp[1] * Ji[k][1] + fp[2] * Ji[k][2]);
    }
    Real r = integrate_lane<Q, HS, HF, Real>(sv, f[0], f[1], f[2], base, ix, iy, iz, sB, sG);
    if (valid) E[(e * C + c) * NQ + qi] = r;
  }
}

// One thread per node: sum the contributions of the (up to 8) elements that
// contain it, in increasing element order.
template <int P, int C>
__global__ void __launch_bounds__(256) structured_scatter_kernel(Grid g, const double* __restrict__ E,
                                                                 double* __restrict__ out) {
  constexpr int n = P + 1;
  constexpr int NPE = n * n * n;
  const int64_t nn = g.Nx * g.Ny * g.Nz;
  const int64_t node = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (node >= nn) return;
  const int64_t I[3] = {node % g.Nx, (node / g.Nx) % g.Ny, node / (g.Nx * g.Ny)};
  const int64_t dims[3] = {g.nx, g.ny, g.nz};
  // per direction: up to two (element index, local index) pairs, lower element first
  int64_t el[3][2];
  int lo[3][2], cnt[3];
  for (int d = 0; d < 3; d++) {
    const int64_t e = I[d] / P;
    const int r = int(I[d] - e * P);
    cnt[d] = 0;
    if (r == 0) {
      if (e > 0) {
        el[d][cnt[d]] = e - 1;
        lo[d][cnt[d]++] = P;
      }
      if (e < dims[d]) {
        el[d][cnt[d]] = e;
        lo[d][cnt[d]++] = 0;
      }
    } else {
      el[d][cnt[d]] = e;
      lo[d][cnt[d]++] = r;
    }
  }
  double acc[C];
#pragma unroll
  for (int c = 0; c < C; c++) acc[c] = 0.0;
  for (int a = 0; a < cnt[2]; a++)
    for (int b = 0; b < cnt[1]; b++)
      for (int k = 0; k < cnt[0]; k++) {
        const int64_t e = el[0][k] + dims[0] * (el[1][b] + dims[1] * el[2][a]);
        const int loc = lo[0][k] + n * (lo[1][b] + n * lo[2][a]);
#pragma unroll
        for (int c = 0; c < C; c++) acc[c] += E[(e * C + c) * NPE + loc];
      }
#pragma unroll
  for (int c = 0; c < C; c++) out[c * nn + node] = acc[c];
}

template <int P, int C, typename State, typename QF>
int run(const Grid& g, const QF& qf, const double* vertices, const double* u, double* r, double t, cudaStream_t s) {
  constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
  constexpr int EPW = 32 / NQ;
  const int64_t ne = int64_t(g.nx) * g.ny * g.nz;
  const int64_t need = ne * C * NQ;
  if (need > kScratchDoubles)
    return sfx_impl::fail(SFX_ERR_UNSUPPORTED,
                          "mesh too large for the no-allocation scratch (" + std::to_string(need) + " doubles needed, " +
                              std::to_string(kScratchDoubles) + " available)");
  double* scratch = nullptr;
  if (int rc = scratch_address(&scratch)) return rc;
  // an error left by earlier, unrelated work is reported as such and left in
  // place for its owner; the checks after each launch then describe this call
  cudaError_t err = cudaPeekAtLastError();
  if (err != cudaSuccess)
    return sfx_impl::fail(SFX_ERR_CUDA, std::string("error pending from earlier work: ") + cudaGetErrorString(err));
  const int64_t warps = (ne + EPW - 1) / EPW;
  const unsigned blocks = unsigned((warps * 32 + 127) / 128);
  structured_residual_kernel<P, C, State, QF><<<blocks, 128, 0, s>>>(g, qf, vertices, u, scratch, t);
  err = cudaGetLastError();
  if (err != cudaSuccess)
    return sfx_impl::fail(SFX_ERR_CUDA, std::string("no-alloc element launch: ") + cudaGetErrorString(err));
  const int64_t nn = g.Nx * g.Ny * g.Nz;
  structured_scatter_kernel<P, C><<<unsigned((nn + 255) / 256), 256, 0, s>>>(g, scratch, r);
  err = cudaGetLastError();
  if (err != cudaSuccess)
    return sfx_impl::fail(SFX_ERR_CUDA, std::string("no-alloc scatter launch: ") + cudaGetErrorString(err));
  return SFX_OK;
}

}  // namespace

extern "C" int sfx_residual_structured_noalloc(int nx, int ny, int nz, int order, int material, const double* params,
                                               const double* vertices, const double* u, double* r, double t,
                                               void* stream) {
  using namespace sfx;
  if (nx < 1 || ny < 1 || nz < 1) return sfx_impl::fail(SFX_ERR_INVALID, "mesh dimensions must be >= 1");
  if (!vertices || !u || !r) return sfx_impl::fail(SFX_ERR_INVALID, "null device pointer");
  if (order != 1 && order != 2) return sfx_impl::fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
  if (!params) return sfx_impl::fail(SFX_ERR_INVALID, "null parameter array");
  Grid g{nx, ny, nz, order, int64_t(order) * nx + 1, int64_t(order) * ny + 1, int64_t(order) * nz + 1};
  auto s = static_cast<cudaStream_t>(stream);
  if (material == SFX_MAT_HEAT) {
    heat_transfer::HeatIntegrand qf{};
    qf.material.conductivity = params[0];
    qf.source = params[1];
    return order == 1 ? run<1, 1, Nothing>(g, qf, vertices, u, r, t, s) : run<2, 1, Nothing>(g, qf, vertices, u, r, t, s);
  }
  if (material == SFX_MAT_NEOHOOKEAN) {
    solid_mechanics::MaterialStressFunctor<solid_mechanics::NeoHookean, true> qf{
        solid_mechanics::NeoHookean{1.0, params[0], params[1]}};
    return order == 1 ? run<1, 3, Empty>(g, qf, vertices, u, r, t, s) : run<2, 3, Empty>(g, qf, vertices, u, r, t, s);
  }
  return sfx_impl::fail(SFX_ERR_UNSUPPORTED, "no-allocation residual supports SFX_MAT_HEAT and SFX_MAT_NEOHOOKEAN");
}
