// Deterministic vector kernels for the Krylov solvers: every reduction is a
// fixed-shape two-pass tree (per-block partial sums in a fixed order, then one
// block reducing the partials in a fixed order), so results are bit-identical
// from run to run.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sfx_blas {

constexpr int kBlock = 256;
constexpr int kMaxPartials = 1024;  // blocks of the first pass

template <typename T>
__device__ inline T block_reduce(T v, T* sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (t < s) sh[t] += sh[t + s];
    __syncthreads();
  }
  T r = sh[0];
  __syncthreads();
  return r;
}

// partial[j * gridDim.x + b] = sum over the block's fixed chunk of x_j . y
// for j = blockIdx.y (grid: blocks x vectors); x_j = X + j * ldx.
// Accumulates in Acc.
template <typename T, typename Acc>
__global__ void __launch_bounds__(kBlock) multi_dot_partial(const T* __restrict__ X, int64_t ldx, int m,
                                                            const T* __restrict__ y, int64_t n,
                                                            Acc* __restrict__ partial) {
  __shared__ Acc sh[kBlock];
  const int j = blockIdx.y;
  if (j >= m) return;
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = int64_t(blockIdx.x) * chunk;
  const int64_t b1 = b0 + chunk < n ? b0 + chunk : n;
  const T* x = X + j * ldx;
  Acc acc = 0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += kBlock) acc += Acc(x[i]) * Acc(y[i]);
  Acc s = block_reduce(acc, sh);
  if (threadIdx.x == 0) partial[int64_t(j) * gridDim.x + blockIdx.x] = s;
}

// out[j] = sum of the nb partials of vector j = blockIdx.x, fixed order
template <typename Acc>
__global__ void __launch_bounds__(kBlock) reduce_partials(const Acc* __restrict__ partial, int nb, int m,
                                                          Acc* __restrict__ out) {
  __shared__ Acc sh[kBlock];
  const int j = blockIdx.x;
  if (j >= m) return;
  Acc acc = 0;
  for (int i = threadIdx.x; i < nb; i += kBlock) acc += partial[int64_t(j) * nb + i];
  Acc s = block_reduce(acc, sh);
  if (threadIdx.x == 0) out[j] = s;
}

// y = a x + b y
template <typename T>
__global__ void axpby(int64_t n, T a, const T* __restrict__ x, T b, T* __restrict__ y) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}

// w -= sum_j h[j] V_j   (h on the device)
template <typename T>
__global__ void multi_axpy_sub(int64_t n, int m, const T* __restrict__ V, int64_t ldv, const T* __restrict__ h,
                               T* __restrict__ w) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T acc = w[i];
  for (int j = 0; j < m; j++) acc -= h[j] * V[j * ldv + i];
  w[i] = acc;
}

// x += sum_j y[j] Z_j  (y on the device)
template <typename T>
__global__ void multi_axpy_add(int64_t n, int m, const T* __restrict__ Z, int64_t ldz, const T* __restrict__ y,
                               T* __restrict__ x) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T acc = x[i];
  for (int j = 0; j < m; j++) acc += y[j] * Z[j * ldz + i];
  x[i] = acc;
}

template <typename T>
__global__ void scale(int64_t n, T a, T* __restrict__ x) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] *= a;
}

// x *= 1 / sqrt(*nrm2) when *nrm2 > 0 (the norm squared stays on the device;
// one thread per block forms the factor)
template <typename T, typename Acc>
__global__ void scale_inv_sqrt(int64_t n, const Acc* __restrict__ nrm2, T* __restrict__ x) {
  __shared__ T a;
  __shared__ bool go;
  if (threadIdx.x == 0) {
    const double v = double(*nrm2);
    go = v > 0.0;
    a = go ? T(1.0 / sqrt(v)) : T(1);
  }
  __syncthreads();
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n && go) x[i] *= a;
}

// z = x / d (elementwise)
template <typename T>
__global__ void diag_solve(int64_t n, const T* __restrict__ x, const T* __restrict__ d, T* __restrict__ z) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) z[i] = x[i] / d[i];
}

// d = a d + b (r / D)
template <typename T>
__global__ void cheb_update(int64_t n, T a, T b, const T* __restrict__ r, const T* __restrict__ D, T* __restrict__ d,
                            T* __restrict__ z) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T v = a * d[i] + b * (r[i] / D[i]);
  d[i] = v;
  z[i] += v;
}

// first Chebyshev step from zero: d = rhs / (theta D), z = d
template <typename T>
__global__ void cheb_start(int64_t n, T inv_theta, const T* __restrict__ rhs, const T* __restrict__ D,
                           T* __restrict__ d, T* __restrict__ z) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T v = rhs[i] / D[i] * inv_theta;
  d[i] = v;
  z[i] = v;
}

// one Chebyshev step with the residual formed in place:
// d = a d + b ((rhs - Jz) / D), z += d
template <typename T>
__global__ void cheb_step(int64_t n, T a, T b, const T* __restrict__ rhs, const T* __restrict__ Jz,
                          const T* __restrict__ D, T* __restrict__ d, T* __restrict__ z) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T v = a * d[i] + b * ((rhs[i] - Jz[i]) / D[i]);
  d[i] = v;
  z[i] += v;
}

// x = a deterministic pseudo-random vector in [-1, 1) (a 64-bit integer hash
// of the index), so that every eigenmode of an operator is present in it
template <typename T>
__global__ void fill_hash(int64_t n, uint64_t seed, T* __restrict__ x) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t h = uint64_t(i) * 0x9E3779B97F4A7C15ull + seed;
  h ^= h >> 30;
  h *= 0xBF58476D1CE4E5B9ull;
  h ^= h >> 27;
  h *= 0x94D049BB133111EBull;
  h ^= h >> 31;
  x[i] = T(double(h >> 11) * (2.0 / 9007199254740992.0) - 1.0);
}

// y = x / sqrt(d)
template <typename T>
__global__ void scale_rsqrt(int64_t n, const T* __restrict__ x, const T* __restrict__ d, T* __restrict__ y) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] / sqrt(d[i]);
}

// Lanczos three-term step: w = w / sqrt(d) - alpha v - beta v_prev is done in
// two kernels: first w /= sqrt(d) (scale_rsqrt in place), then this one
template <typename T>
__global__ void lanczos_orth(int64_t n, T alpha, const T* __restrict__ v, T beta, const T* __restrict__ vp,
                             T* __restrict__ w) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) w[i] = w[i] - alpha * v[i] - beta * vp[i];
}

// ------------------------------------------------ device-side GMRES(m) state
// Least-squares state of one GMRES cycle kept on the device, so that a whole
// cycle can run as one CUDA graph without reading anything back:
//   st[0] beta = |r0|, st[1] target, st[2] steps taken (k_done, as a double),
//   g[m + 1], cs[m], sn[m], H column-major [m][m + 1].
struct GmresLayout {
  int m;
  __host__ __device__ int64_t size() const { return 3 + (m + 1) + 2 * m + int64_t(m + 1) * m; }
  __host__ __device__ double* g(double* st) const { return st + 3; }
  __host__ __device__ double* cs(double* st) const { return st + 3 + (m + 1); }
  __host__ __device__ double* sn(double* st) const { return st + 3 + (m + 1) + m; }
  __host__ __device__ double* H(double* st) const { return st + 3 + (m + 1) + 2 * m; }
};

// beta = sqrt(*nrm2), g = beta e_1, target = max(rel beta, abs); no step taken yet
template <typename Acc>
__global__ void gmres_init(GmresLayout L, const Acc* __restrict__ nrm2, double rel, double abs_tol,
                           double* __restrict__ st) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double beta = sqrt(double(*nrm2) > 0.0 ? double(*nrm2) : 0.0);
  st[0] = beta;
  st[1] = fmax(rel * beta, abs_tol);
  st[2] = beta > 0.0 ? -1.0 : 0.0;  // -1: running; >= 0: steps kept
  double* g = L.g(st);
  for (int i = 0; i <= L.m; i++) g[i] = 0.0;
  g[0] = beta;
}

// Arnoldi column k from the two Gram-Schmidt passes (c1, c2: k + 1
// coefficients each) and the new vector's squared norm c3, then the Givens
// rotations (Saad, Alg. 6.9): previous rotations applied, a new one formed,
// the residual estimate |g[k+1]| updated.  The cycle stops counting once the
// estimate reaches the target (or the new vector vanishes, or k = m - 1).
template <typename Acc>
__global__ void gmres_step(GmresLayout L, int k, const Acc* __restrict__ c1, const Acc* __restrict__ c2,
                           const Acc* __restrict__ c3, double* __restrict__ st) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (st[2] >= 0.0) return;  // converged earlier (or zero right-hand side)
  double* Hk = L.H(st) + int64_t(k) * (L.m + 1);
  double* cs = L.cs(st);
  double* sn = L.sn(st);
  double* g = L.g(st);
  for (int j = 0; j <= k; j++) Hk[j] = double(c1[j]) + double(c2[j]);
  const double hn = sqrt(double(*c3) > 0.0 ? double(*c3) : 0.0);
  Hk[k + 1] = hn;
  for (int j = 0; j < k; j++) {
    const double t = cs[j] * Hk[j] + sn[j] * Hk[j + 1];
    Hk[j + 1] = -sn[j] * Hk[j] + cs[j] * Hk[j + 1];
    Hk[j] = t;
  }
  double d = hypot(Hk[k], Hk[k + 1]);
  if (d == 0.0) d = 1e-300;
  cs[k] = Hk[k] / d;
  sn[k] = Hk[k + 1] / d;
  Hk[k] = d;
  Hk[k + 1] = 0.0;
  g[k + 1] = -sn[k] * g[k];
  g[k] = cs[k] * g[k];
  if (fabs(g[k + 1]) <= st[1] || hn == 0.0 || k == L.m - 1) st[2] = double(k + 1);
}

// y = H^-1 g over the steps kept (zero beyond them); adds them to *count
template <typename T>
__global__ void gmres_solve(GmresLayout L, double* __restrict__ st, T* __restrict__ y, int* __restrict__ count) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int k = st[2] > 0.0 ? int(st[2]) : 0;
  const double* H = L.H(st);
  const double* g = L.g(st);
  double yv[256];
  for (int i = k - 1; i >= 0; i--) {
    double acc = g[i];
    for (int j = i + 1; j < k; j++) acc -= H[int64_t(j) * (L.m + 1) + i] * yv[j];
    yv[i] = acc / H[int64_t(i) * (L.m + 1) + i];
  }
  for (int i = 0; i < L.m; i++) y[i] = i < k ? T(yv[i]) : T(0);
  *count += k;
}

template <typename S, typename T>
__global__ void convert(int64_t n, const S* __restrict__ x, T* __restrict__ y) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = T(x[i]);
}

// x[idx[k]] = v[k] or value
template <typename T>
__global__ void set_entries(int64_t m, const int64_t* __restrict__ idx, T value, T* __restrict__ x) {
  int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m) x[idx[k]] = value;
}
template <typename T>
__global__ void copy_entries(int64_t m, const int64_t* __restrict__ idx, const T* __restrict__ src, T* __restrict__ x) {
  int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m) x[idx[k]] = src[idx[k]];
}

// x[idx[k]] = a[idx[k]] - b[idx[k]]
template <typename T>
__global__ void diff_entries(int64_t m, const int64_t* __restrict__ idx, const T* __restrict__ a,
                             const T* __restrict__ b, T* __restrict__ x) {
  int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < m) x[idx[k]] = a[idx[k]] - b[idx[k]];
}

// r = b - r (in place on r)
template <typename T>
__global__ void rsub(int64_t n, const T* __restrict__ b, T* __restrict__ r) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) r[i] = b[i] - r[i];
}

// nonzero count of non-finite entries (flag)
template <typename T>
__global__ void nonfinite_flag(int64_t n, const T* __restrict__ x, int* __restrict__ flag) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n && !isfinite(double(x[i]))) *flag = 1;
}

}  // namespace sfx_blas
