// Device-resident Newton-Krylov solver over an sfx form.
//
// Newton (serac's NewtonSolver without line search, equation_solver.cpp:79-200):
//   r = R(u), r[ess] = 0; until ||r|| <= max(rel ||r0||, abs):
//     linearise at u (stored tangent), solve J du = r, u -= du
// Krylov: right-preconditioned restarted GMRES(m) / flexible GMRES (Saad,
// Iterative Methods, Alg. 6.9 / 9.5) with classical Gram-Schmidt applied
// twice, or Jacobi-preconditioned CG (Alg. 6.18) for symmetric problems.
// Preconditioners: Jacobi, Jacobi-Chebyshev (Chebyshev iteration on D^-1 J
// over [lmax/ratio, 1.05 lmax], lmax from a Lanczos estimate), and, in the
// mixed-precision mode, an inner FP32 GMRES(k) on the FP32 stored tangent with
// FP32 Jacobi-Chebyshev inside FP64 flexible GMRES.
// Dirichlet rows/columns: J[ess, :] = J[:, ess] = I on the essential set,
// residual entries zeroed (solid_mechanics.hpp:1118-1139).
// Vectors and reductions stay on the device; the host reads back only the
// Gram-Schmidt coefficients of each Krylov step (deterministic tree sums).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "blas.cuh"
#include "form.hpp"
#include "learned_internal.hpp"
#include "sfx.h"
#include "sfx_solver.h"

using namespace sfx_impl;

namespace {

inline unsigned nblocks(int64_t n, int b = 256) { return unsigned((n + b - 1) / b); }

template <typename T>
struct Vec {
  DeviceBuf<T> buf;
  T* p() const { return buf.p; }
};

template <typename T, typename Acc>
struct Reducer {
  DeviceBuf<Acc> partial;
  DeviceBuf<Acc> out;
  DeviceBuf<Acc> coef;  // Gram-Schmidt coefficients of both passes and the norm, read back together
  Acc* pinned = nullptr;  // their host copy (page-locked, so the read-back can sit in a CUDA graph)
  std::vector<Acc> host;
  int nb = 0;
  Reducer() = default;
  Reducer(const Reducer&) = delete;
  Reducer& operator=(const Reducer&) = delete;
  ~Reducer() {
    if (pinned) cudaFreeHost(pinned);
  }
  cudaError_t init(int64_t n, int max_m) {
    nb = int(std::min<int64_t>(sfx_blas::kMaxPartials, std::max<int64_t>(1, (n + 4095) / 4096)));
    cudaError_t e = partial.alloc(size_t(nb) * max_m);
    if (e == cudaSuccess) e = out.alloc(size_t(max_m));
    if (e == cudaSuccess) e = coef.alloc(size_t(2 * max_m + 1));
    if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&pinned), sizeof(Acc) * size_t(2 * max_m + 1), 0);
    host.resize(size_t(2 * max_m + 1));
    return e;
  }
  // host[j] = X_j . y for j < m (one synchronisation)
  cudaError_t multi_dot(const T* X, int64_t ldx, int m, const T* y, int64_t n, cudaStream_t s) {
    sfx_blas::multi_dot_partial<T, Acc><<<dim3(nb, m), sfx_blas::kBlock, 0, s>>>(X, ldx, m, y, n, partial.p);
    sfx_blas::reduce_partials<Acc><<<m, sfx_blas::kBlock, 0, s>>>(partial.p, nb, m, out.p);
    cudaError_t e = cudaMemcpyAsync(host.data(), out.p, sizeof(Acc) * m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
  }
  Acc dot(const T* x, const T* y, int64_t n, cudaStream_t s, cudaError_t* err) {
    *err = multi_dot(x, 0, 1, y, n, s);
    return host[0];
  }
  // dst[j] = X_j . y on the device, no synchronisation
  void multi_dot_to(const T* X, int64_t ldx, int m, const T* y, int64_t n, Acc* dst, cudaStream_t s) {
    sfx_blas::multi_dot_partial<T, Acc><<<dim3(nb, m), sfx_blas::kBlock, 0, s>>>(X, ldx, m, y, n, partial.p);
    sfx_blas::reduce_partials<Acc><<<m, sfx_blas::kBlock, 0, s>>>(partial.p, nb, m, dst);
  }
};

}  // namespace

struct sfx_solver_s {
  sfx_form form = nullptr;
  sfx_solver_options opt{};
  sfx_solver_stats stats{};
  int64_t n = 0;
  DeviceBuf<int64_t> ess;
  int64_t n_ess = 0;
  bool transpose = false;  // linear solves with J^T (adjoint problems)
  // FP64 work vectors
  DeviceBuf<double> r, du, tmp, tmp2, diag, cheb_d, cheb_r, V, Z, y, wx;
  // FP32 work vectors
  DeviceBuf<float> diag32, x32, b32, tmp32, tmp32b, cheb_d32, cheb_r32, V32, y32;
  Reducer<double, double> red;
  Reducer<float, float> red32;
  double lmax = 0.0, lmax32 = 0.0;
  int nn_rejected_run = 0;  // network steps skipped in a row in the current linear solve
  // learned preconditioner
  sfx_lnet net = nullptr;
  int grid[3] = {0, 0, 0};
  const float* features = nullptr;
  DeviceBuf<float> nn_z, nn_res, nn_x, x32b;
  // the inner FP32 GMRES cycle as one CUDA graph, captured on a private
  // stream and valid for one linear solve (it holds that solve's Chebyshev
  // coefficients); its least-squares state and iteration count stay on the device
  cudaStream_t capture = nullptr;
  cudaGraphExec_t inner_graph = nullptr;
  DeviceBuf<double> gstate;
  DeviceBuf<int> inner_count;
  void drop_graphs() {
    if (inner_graph) cudaGraphExecDestroy(inner_graph);
    inner_graph = nullptr;
  }
  ~sfx_solver_s() {
    drop_graphs();
    if (capture) cudaStreamDestroy(capture);
  }
};

namespace {

// ---------------------------------------------------------------- operators
int apply_J64(sfx_solver s, const double* x, double* y, cudaStream_t st) {
  // y = P J P x with P the projection onto the free vdofs; every vector the
  // solvers pass in is already zero on the essential set (P x = x), so only
  // the output rows need zeroing
  if (int rc = s->transpose ? sfx_jvp_transpose(s->form, x, y, st) : sfx_jvp(s->form, x, y, st)) return rc;
  if (s->n_ess) sfx_blas::set_entries<double><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 0.0, y);
  return SFX_OK;
}

int apply_J32(sfx_solver s, const float* x, float* y, cudaStream_t st) {
  if (int rc = s->transpose ? sfx_jvp_transpose_f32(s->form, x, y, st) : sfx_jvp_f32(s->form, x, y, st)) return rc;
  if (s->n_ess) sfx_blas::set_entries<float><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 0.0f, y);
  return SFX_OK;
}

// degree of the FP32 Chebyshev polynomial inside the mixed-precision solve
int inner_degree(sfx_solver s) {
  return s->opt.inner_chebyshev_degree > 0 ? s->opt.inner_chebyshev_degree : s->opt.chebyshev_degree;
}

// Eigenvalues of the symmetric tridiagonal matrix (diagonal a, off-diagonal
// b[1..m-1]) and the last component of each normalised eigenvector, by cyclic
// Jacobi rotations on the dense m x m matrix (m is a few tens).
void tridiagonal_eigen(const std::vector<double>& a, const std::vector<double>& b, std::vector<double>& lam,
                       std::vector<double>& last) {
  const int m = int(a.size());
  std::vector<double> A(size_t(m) * m, 0.0), Vm(size_t(m) * m, 0.0);
  for (int i = 0; i < m; i++) {
    A[size_t(i) * m + i] = a[size_t(i)];
    Vm[size_t(i) * m + i] = 1.0;
    if (i > 0) A[size_t(i) * m + i - 1] = A[size_t(i - 1) * m + i] = b[size_t(i)];
  }
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0.0;
    for (int p = 0; p < m; p++)
      for (int q = p + 1; q < m; q++) off += A[size_t(p) * m + q] * A[size_t(p) * m + q];
    if (off < 1e-30) break;
    for (int p = 0; p < m; p++)
      for (int q = p + 1; q < m; q++) {
        const double apq = A[size_t(p) * m + q];
        if (apq == 0.0) continue;
        const double th = 0.5 * (A[size_t(q) * m + q] - A[size_t(p) * m + p]) / apq;
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < m; k++) {  // columns p, q
          const double akp = A[size_t(k) * m + p], akq = A[size_t(k) * m + q];
          A[size_t(k) * m + p] = c * akp - sn * akq;
          A[size_t(k) * m + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < m; k++) {  // rows p, q
          const double apk = A[size_t(p) * m + k], aqk = A[size_t(q) * m + k];
          A[size_t(p) * m + k] = c * apk - sn * aqk;
          A[size_t(q) * m + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < m; k++) {
          const double vkp = Vm[size_t(k) * m + p], vkq = Vm[size_t(k) * m + q];
          Vm[size_t(k) * m + p] = c * vkp - sn * vkq;
          Vm[size_t(k) * m + q] = sn * vkp + c * vkq;
        }
      }
  }
  lam.resize(size_t(m));
  last.resize(size_t(m));
  for (int i = 0; i < m; i++) {
    lam[size_t(i)] = A[size_t(i) * m + i];
    last[size_t(i)] = Vm[size_t(m - 1) * m + i];
  }
}

// Upper estimate of the largest eigenvalue of D^-1 J.  For symmetric J the
// operator is self-adjoint in the D inner product, so Lanczos runs on
// A = D^-1/2 J D^-1/2 (Saad, Iterative Methods, Alg. 6.15) from a
// deterministic pseudo-random start (every mode present: a smooth start
// would hide the high-frequency modes that set lmax), for
// opt.eigen_iterations steps; the estimate is the largest Ritz value plus its
// residual |beta_{m+1} s_m|, which bounds its distance to an eigenvalue.
template <typename T, typename Acc>
int estimate_lmax(sfx_solver s, int (*apply)(sfx_solver, const T*, T*, cudaStream_t), const T* D, T* v, T* w,
                  T* vp, T* t, Reducer<T, Acc>& red, double* lmax, cudaStream_t st) {
  const int64_t n = s->n;
  const int m = std::max(2, s->opt.eigen_iterations);
  cudaError_t err;
  sfx_blas::fill_hash<T><<<nblocks(n), 256, 0, st>>>(n, 0x5eed5eedull, v);
  if (s->n_ess) sfx_blas::set_entries<T><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, T(0), v);
  SFX_CUDA_TRY(cudaMemsetAsync(vp, 0, sizeof(T) * n, st));
  {
    const double nv = std::sqrt(double(red.dot(v, v, n, st, &err)));
    SFX_CUDA_TRY(err);
    sfx_blas::scale<T><<<nblocks(n), 256, 0, st>>>(n, T(1.0 / nv), v);
  }
  std::vector<double> alpha, beta(1, 0.0);
  double beta_next = 0.0;
  for (int j = 0; j < m; j++) {
    sfx_blas::scale_rsqrt<T><<<nblocks(n), 256, 0, st>>>(n, v, D, t);
    if (int rc = apply(s, t, w, st)) return rc;
    sfx_blas::scale_rsqrt<T><<<nblocks(n), 256, 0, st>>>(n, w, D, w);
    const double a = double(red.dot(w, v, n, st, &err));
    SFX_CUDA_TRY(err);
    if (!std::isfinite(a)) return fail(SFX_ERR_NONFINITE, "non-finite Lanczos coefficient");
    alpha.push_back(a);
    sfx_blas::lanczos_orth<T><<<nblocks(n), 256, 0, st>>>(n, T(a), v, T(beta.back()), vp, w);
    beta_next = std::sqrt(double(red.dot(w, w, n, st, &err)));
    SFX_CUDA_TRY(err);
    if (!(beta_next > 1e-14 * std::fabs(a)) || j == m - 1) break;  // invariant subspace found, or done
    beta.push_back(beta_next);
    std::swap(vp, v);  // vp <- v
    std::swap(v, w);   // v <- w / beta
    sfx_blas::scale<T><<<nblocks(n), 256, 0, st>>>(n, T(1.0 / beta_next), v);
  }
  std::vector<double> lam, last;
  tridiagonal_eigen(alpha, beta, lam, last);
  size_t imax = 0;
  for (size_t i = 1; i < lam.size(); i++)
    if (lam[i] > lam[imax]) imax = i;
  *lmax = lam[imax] + std::fabs(beta_next * last[imax]);
  s->stats.lmax_estimate = *lmax;
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

// z = Chebyshev(D^-1 J) approximation of J^-1 b, degree k, starting from 0
template <typename T, typename Acc>
int chebyshev(sfx_solver s, int (*apply)(sfx_solver, const T*, T*, cudaStream_t), const T* D, double lmax,
              int degree, double ratio, const T* b, T* z, T* d, T* res, cudaStream_t st) {
  const int64_t n = s->n;
  const double hi = 1.05 * lmax, lo = lmax / ratio;
  const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  // d = D^-1 b / theta ; z = d
  sfx_blas::cheb_start<T><<<nblocks(n), 256, 0, st>>>(n, T(1.0 / theta), b, D, d, z);
  for (int k = 1; k < degree; k++) {
    if (int rc = apply(s, z, res, st)) return rc;  // res = J z
    double rho_new = 1.0 / (2.0 * sigma - rho);
    sfx_blas::cheb_step<T><<<nblocks(n), 256, 0, st>>>(n, T(rho_new * rho), T(2.0 * rho_new / delta), b, res, D, d, z);
    rho = rho_new;
  }
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

// Restarted right-preconditioned (flexible) GMRES on vectors of type T with
// accumulation type Acc.  x holds the initial guess and the result.
template <typename T, typename Acc>
int gmres(sfx_solver s, int (*apply)(sfx_solver, const T*, T*, cudaStream_t),
          const std::function<int(const T*, T*, cudaStream_t)>& precond, bool flexible, const T* b, T* x, T* V,
          T* Zs, T* w, T* ydev, Reducer<T, Acc>& red, int restart, int max_iters, double rel_tol, double abs_tol,
          int* iters_out, double* rel_out, cudaStream_t st) {
  const int64_t n = s->n;
  cudaError_t err;
  const double nb = std::sqrt(double(red.dot(b, b, n, st, &err)));
  SFX_CUDA_TRY(err);
  *iters_out = 0;
  if (nb == 0.0) {
    SFX_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(T) * n, st));
    *rel_out = 0.0;
    return SFX_OK;
  }
  const double target = std::max(rel_tol * nb, abs_tol);
  int total = 0;
  const size_t mr = static_cast<size_t>(restart);
  std::vector<double> H((mr + 1) * mr), cs(mr), sn(mr), g(mr + 1), yv(mr);
  std::vector<T> yh(mr + 1);
  double beta = 0.0;
  while (true) {
    // r = b - A x into V_0
    if (int rc = apply(s, x, V, st)) return rc;
    sfx_blas::rsub<T><<<nblocks(n), 256, 0, st>>>(n, b, V);
    beta = std::sqrt(double(red.dot(V, V, n, st, &err)));
    SFX_CUDA_TRY(err);
    if (!std::isfinite(beta)) return fail(SFX_ERR_NONFINITE, "non-finite residual in GMRES");
    if (beta <= target || total >= max_iters) break;
    sfx_blas::scale<T><<<nblocks(n), 256, 0, st>>>(n, T(1.0 / beta), V);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    bool done = false;
    for (k = 0; k < restart && total < max_iters; k++) {
      T* vk = V + int64_t(k) * n;
      T* zk = flexible ? Zs + int64_t(k) * n : w;
      T* vnext = V + int64_t(k + 1) * n;
      // one Arnoldi step: precondition, apply, classical Gram-Schmidt twice,
      // normalise; the coefficients and the norm stay on the device and are
      // read back once (page-locked buffer)
      static_assert(std::is_same<T, Acc>::value, "coefficients are applied in the vector type");
      Acc* c1 = red.coef.p;
      Acc* c2 = red.coef.p + (k + 1);
      Acc* c3 = red.coef.p + 2 * (k + 1);
      const size_t ncoef = size_t(2 * (k + 1) + 1);
      auto step = [&](cudaStream_t ss) -> int {
        if (int rc = precond(vk, zk, ss)) return rc;
        if (int rc = apply(s, zk, vnext, ss)) return rc;
        red.multi_dot_to(V, n, k + 1, vnext, n, c1, ss);
        sfx_blas::multi_axpy_sub<T><<<nblocks(n), 256, 0, ss>>>(n, k + 1, V, n, c1, vnext);
        red.multi_dot_to(V, n, k + 1, vnext, n, c2, ss);
        sfx_blas::multi_axpy_sub<T><<<nblocks(n), 256, 0, ss>>>(n, k + 1, V, n, c2, vnext);
        red.multi_dot_to(vnext, 0, 1, vnext, n, c3, ss);
        sfx_blas::scale_inv_sqrt<T, Acc><<<nblocks(n), 256, 0, ss>>>(n, c3, vnext);
        SFX_CUDA_TRY(cudaMemcpyAsync(red.pinned, red.coef.p, sizeof(Acc) * ncoef, cudaMemcpyDeviceToHost, ss));
        SFX_CUDA_TRY(cudaGetLastError());
        return SFX_OK;
      };
      if (int rc = step(st)) return rc;
      SFX_CUDA_TRY(cudaStreamSynchronize(st));
      double* Hk = &H[size_t(k) * (restart + 1)];
      for (int j = 0; j <= k; j++) Hk[j] = double(red.pinned[size_t(j)]) + double(red.pinned[size_t(k + 1 + j)]);
      double hn = std::sqrt(double(red.pinned[size_t(2 * (k + 1))]));
      Hk[k + 1] = hn;
      for (int j = 0; j < k; j++) {
        double t = cs[size_t(j)] * Hk[j] + sn[size_t(j)] * Hk[j + 1];
        Hk[j + 1] = -sn[size_t(j)] * Hk[j] + cs[size_t(j)] * Hk[j + 1];
        Hk[j] = t;
      }
      double d = std::hypot(Hk[k], Hk[k + 1]);
      if (d == 0.0) d = 1e-300;
      cs[size_t(k)] = Hk[k] / d;
      sn[size_t(k)] = Hk[k + 1] / d;
      Hk[k] = d;
      Hk[k + 1] = 0.0;
      g[size_t(k + 1)] = -sn[size_t(k)] * g[size_t(k)];
      g[size_t(k)] = cs[size_t(k)] * g[size_t(k)];
      total++;
      if (std::fabs(g[size_t(k + 1)]) <= target || hn == 0.0) {
        k++;
        done = true;
        break;
      }
    }
    if (!done) k = std::min(k, restart);
    // back substitution H y = g
    for (int i = k - 1; i >= 0; i--) {
      double acc = g[size_t(i)];
      for (int j = i + 1; j < k; j++) acc -= H[size_t(j) * (restart + 1) + i] * yv[size_t(j)];
      yv[size_t(i)] = acc / H[size_t(i) * (restart + 1) + i];
    }
    for (int i = 0; i < k; i++) yh[size_t(i)] = T(yv[size_t(i)]);
    SFX_CUDA_TRY(cudaMemcpyAsync(ydev, yh.data(), sizeof(T) * k, cudaMemcpyHostToDevice, st));
    if (flexible) {
      sfx_blas::multi_axpy_add<T><<<nblocks(n), 256, 0, st>>>(n, k, Zs, n, ydev, x);
    } else {
      // x += M (V y): form V y in w, precondition into V_k slot (free), add
      SFX_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(T) * n, st));
      sfx_blas::multi_axpy_add<T><<<nblocks(n), 256, 0, st>>>(n, k, V, n, ydev, w);
      T* zz = V + int64_t(k) * n;
      if (int rc = precond(w, zz, st)) return rc;
      sfx_blas::axpby<T><<<nblocks(n), 256, 0, st>>>(n, T(1), zz, T(1), x);
    }
    SFX_CUDA_TRY(cudaGetLastError());
    if (done && total >= max_iters) {
      // fall through to the true-residual check
    }
  }
  *iters_out = total;
  *rel_out = beta / nb;
  return SFX_OK;
}

// One cycle of the inner FP32 GMRES(m) with x0 = 0 (right-preconditioned by
// FP32 Jacobi-Chebyshev), x = M V y: Arnoldi with classical Gram-Schmidt
// applied twice and the Givens least-squares update on the device
// (gmres_step), so the whole cycle - m preconditioner and operator
// applications - is captured once per linear solve as one CUDA graph and
// replayed by every outer step without a host round trip.  The residual
// estimate ends the counting of steps at inner_rel_tol; the steps after it
// still run (their coefficients are not used).
int inner_gmres(sfx_solver s, const float* b, float* x, cudaStream_t st) {
  const int64_t n = s->n;
  const int m = s->opt.inner_iterations;
  const sfx_blas::GmresLayout L{m};
  if (!s->inner_graph) {
    auto body = [&](cudaStream_t ss) -> int {
      float* V = s->V32.p;
      float* c1 = s->red32.coef.p;
      SFX_CUDA_TRY(cudaMemcpyAsync(V, b, sizeof(float) * n, cudaMemcpyDeviceToDevice, ss));
      s->red32.multi_dot_to(V, 0, 1, V, n, c1, ss);
      sfx_blas::gmres_init<float><<<1, 1, 0, ss>>>(L, c1, s->opt.inner_rel_tol, 0.0, s->gstate.p);
      sfx_blas::scale_inv_sqrt<float, float><<<nblocks(n), 256, 0, ss>>>(n, c1, V);
      for (int k = 0; k < m; k++) {
        float* vk = V + int64_t(k) * n;
        float* vnext = V + int64_t(k + 1) * n;
        float* k1 = s->red32.coef.p;
        float* k2 = k1 + (k + 1);
        float* k3 = k1 + 2 * (k + 1);
        if (int rc = chebyshev<float, float>(s, apply_J32, s->diag32.p, s->lmax32, inner_degree(s),
                                             s->opt.chebyshev_ratio, vk, s->tmp32.p, s->cheb_d32.p, s->cheb_r32.p, ss))
          return rc;
        if (int rc = apply_J32(s, s->tmp32.p, vnext, ss)) return rc;
        s->red32.multi_dot_to(V, n, k + 1, vnext, n, k1, ss);
        sfx_blas::multi_axpy_sub<float><<<nblocks(n), 256, 0, ss>>>(n, k + 1, V, n, k1, vnext);
        s->red32.multi_dot_to(V, n, k + 1, vnext, n, k2, ss);
        sfx_blas::multi_axpy_sub<float><<<nblocks(n), 256, 0, ss>>>(n, k + 1, V, n, k2, vnext);
        s->red32.multi_dot_to(vnext, 0, 1, vnext, n, k3, ss);
        sfx_blas::scale_inv_sqrt<float, float><<<nblocks(n), 256, 0, ss>>>(n, k3, vnext);
        sfx_blas::gmres_step<float><<<1, 1, 0, ss>>>(L, k, k1, k2, k3, s->gstate.p);
      }
      sfx_blas::gmres_solve<float><<<1, 1, 0, ss>>>(L, s->gstate.p, s->y32.p, s->inner_count.p);
      SFX_CUDA_TRY(cudaMemsetAsync(s->tmp32b.p, 0, sizeof(float) * n, ss));
      sfx_blas::multi_axpy_add<float><<<nblocks(n), 256, 0, ss>>>(n, m, V, n, s->y32.p, s->tmp32b.p);
      if (int rc = chebyshev<float, float>(s, apply_J32, s->diag32.p, s->lmax32, inner_degree(s),
                                           s->opt.chebyshev_ratio, s->tmp32b.p, x, s->cheb_d32.p, s->cheb_r32.p, ss))
        return rc;
      SFX_CUDA_TRY(cudaGetLastError());
      return SFX_OK;
    };
    SFX_CUDA_TRY(cudaStreamBeginCapture(s->capture, cudaStreamCaptureModeThreadLocal));
    const int rc = body(s->capture);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->capture, &graph);
    if (rc || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return rc ? rc : fail(SFX_ERR_CUDA, std::string("inner cycle capture: ") + cudaGetErrorString(e));
    }
    const cudaError_t ei = cudaGraphInstantiate(&s->inner_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      s->inner_graph = nullptr;
      return fail(SFX_ERR_CUDA, std::string("inner cycle graph: ") + cudaGetErrorString(ei));
    }
  }
  SFX_CUDA_TRY(cudaGraphLaunch(s->inner_graph, st));
  return SFX_OK;
}

// Jacobi-preconditioned CG (symmetric positive definite J)
int cg(sfx_solver s, const double* b, double* x, int* iters_out, double* rel_out, cudaStream_t st) {
  const int64_t n = s->n;
  cudaError_t err;
  double* r = s->V.p;
  double* z = s->V.p + n;
  double* p = s->V.p + 2 * n;
  double* q = s->V.p + 3 * n;
  SFX_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
  SFX_CUDA_TRY(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  const double nb = std::sqrt(s->red.dot(b, b, n, st, &err));
  SFX_CUDA_TRY(err);
  *iters_out = 0;
  *rel_out = 0.0;
  if (nb == 0.0) return SFX_OK;
  const double target = std::max(s->opt.krylov_rel_tol * nb, s->opt.krylov_abs_tol);
  sfx_blas::diag_solve<double><<<nblocks(n), 256, 0, st>>>(n, r, s->diag.p, z);
  SFX_CUDA_TRY(cudaMemcpyAsync(p, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  double rz = s->red.dot(r, z, n, st, &err);
  SFX_CUDA_TRY(err);
  double rn = nb;
  int it = 0;
  for (it = 1; it <= s->opt.max_krylov_iterations; it++) {
    if (int rc = apply_J64(s, p, q, st)) return rc;
    double pq = s->red.dot(p, q, n, st, &err);
    SFX_CUDA_TRY(err);
    if (!(pq > 0.0)) return fail(SFX_ERR_NONFINITE, "CG breakdown (operator not positive definite)");
    double alpha = rz / pq;
    sfx_blas::axpby<double><<<nblocks(n), 256, 0, st>>>(n, alpha, p, 1.0, x);
    sfx_blas::axpby<double><<<nblocks(n), 256, 0, st>>>(n, -alpha, q, 1.0, r);
    rn = std::sqrt(s->red.dot(r, r, n, st, &err));
    SFX_CUDA_TRY(err);
    if (rn <= target) break;
    sfx_blas::diag_solve<double><<<nblocks(n), 256, 0, st>>>(n, r, s->diag.p, z);
    double rz_new = s->red.dot(r, z, n, st, &err);
    SFX_CUDA_TRY(err);
    sfx_blas::axpby<double><<<nblocks(n), 256, 0, st>>>(n, 1.0, z, rz_new / rz, p);
    rz = rz_new;
  }
  *iters_out = std::min(it, s->opt.max_krylov_iterations);
  *rel_out = rn / nb;
  return SFX_OK;
}

int ensure(DeviceBuf<double>& b, size_t n) { return b.n >= n ? SFX_OK : (b.alloc(n) == cudaSuccess ? SFX_OK : SFX_ERR_NOMEM); }
int ensure(DeviceBuf<float>& b, size_t n) { return b.n >= n ? SFX_OK : (b.alloc(n) == cudaSuccess ? SFX_OK : SFX_ERR_NOMEM); }

// one linear solve J du = r at the current linearisation
int linear_solve(sfx_solver s, const double* rhs, double* x, cudaStream_t st) {
  const int64_t n = s->n;
  const auto& o = s->opt;
  int iters = 0;
  double rel = 0.0;
  // graphs of the inner steps hold the previous linearisation's Chebyshev coefficients
  s->drop_graphs();
  // Jacobi diagonal with unit entries on the essential set
  if (int rc = sfx_assemble_diagonal(s->form, s->diag.p, st)) return rc;
  if (s->n_ess) sfx_blas::set_entries<double><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 1.0, s->diag.p);
  if (o.krylov == SFX_KRYLOV_CG) {
    int rc = cg(s, rhs, x, &iters, &rel, st);
    s->stats.krylov_iterations += iters;
    s->stats.last_krylov_rel = rel;
    return rc;
  }
  const int m = o.restart;
  if (ensure(s->V, size_t(m + 1) * n) || ensure(s->Z, size_t(m) * n))
    return fail(SFX_ERR_NOMEM, "Krylov basis allocation failed");
  // the outer preconditioner runs on st (it is not captured); the stream argument is unused
  std::function<int(const double*, double*, cudaStream_t)> prec;
  if (o.precond == SFX_PREC_NONE) {
    prec = [=](const double* v, double* z, cudaStream_t) -> int {
      SFX_CUDA_TRY(cudaMemcpyAsync(z, v, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      return SFX_OK;
    };
  } else if (o.precond == SFX_PREC_JACOBI) {
    prec = [=](const double* v, double* z, cudaStream_t) -> int {
      sfx_blas::diag_solve<double><<<nblocks(n), 256, 0, st>>>(n, v, s->diag.p, z);
      return SFX_OK;
    };
  } else if (o.precond == SFX_PREC_LEARNED) {
    if (!s->net || !s->features) return fail(SFX_ERR_INVALID, "SFX_PREC_LEARNED needs sfx_solver_set_learned");
    const int k = o.inner_iterations;
    if (ensure(s->x32, n) || ensure(s->b32, n) || ensure(s->tmp32, n) || ensure(s->diag32, n) ||
        ensure(s->cheb_d32, n) || ensure(s->cheb_r32, n) || ensure(s->tmp32b, n) || ensure(s->nn_z, n) ||
        ensure(s->nn_res, n) || ensure(s->nn_x, n) || ensure(s->x32b, n) ||
        (o.mixed_precision && (ensure(s->V32, size_t(k + 1) * n) || ensure(s->y32, size_t(k + 1)))))
      return fail(SFX_ERR_NOMEM, "FP32 workspace allocation failed");
    sfx_blas::convert<double, float><<<nblocks(n), 256, 0, st>>>(n, s->diag.p, s->diag32.p);
    if (int rc = estimate_lmax<float, float>(s, apply_J32, s->diag32.p, s->tmp32.p, s->cheb_r32.p, s->cheb_d32.p,
                                             s->tmp32b.p, s->red32, &s->lmax32, st))
      return rc;
    // Network step on the residual res: z += a NN(res) with a minimising
    // |res - a J NN(res)|, kept only when it takes at least 1 % off the
    // residual norm (otherwise skipped: a fallback).  Returns what is left
    // of the residual (nn_res, or res itself after a fallback).
    auto nn_step = [=](const float* res, float* z, const float** left) -> int {
      cudaError_t err;
      *left = res;
      if (o.learned_max_rejections > 0 && s->nn_rejected_run >= o.learned_max_rejections) {
        s->stats.learned_skipped++;  // the network kept failing in this linear solve
        return SFX_OK;
      }
      const double nv = double(s->red32.dot(res, res, n, st, &err));
      SFX_CUDA_TRY(err);
      if (int rc = lnet_apply(s->net, s->grid[0], s->grid[1], s->grid[2], res, s->features, s->nn_z.p, st)) return rc;
      if (s->n_ess) sfx_blas::set_entries<float><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 0.0f, s->nn_z.p);
      s->stats.learned_applications++;
      if (int rc = apply_J32(s, s->nn_z.p, s->nn_x.p, st)) return rc;
      const double rj = double(s->red32.dot(res, s->nn_x.p, n, st, &err));
      SFX_CUDA_TRY(err);
      const double jj = double(s->red32.dot(s->nn_x.p, s->nn_x.p, n, st, &err));
      SFX_CUDA_TRY(err);
      const double a = jj > 0.0 ? rj / jj : 0.0;
      const double nr = nv - a * rj;  // |res - a J NN(res)|^2
      if (std::isfinite(a) && std::isfinite(jj) && jj > 0.0 && nr <= 0.9801 * nv) {
        sfx_blas::axpby<float><<<nblocks(n), 256, 0, st>>>(n, float(a), s->nn_z.p, 1.0f, z);
        SFX_CUDA_TRY(cudaMemcpyAsync(s->nn_res.p, res, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
        sfx_blas::axpby<float><<<nblocks(n), 256, 0, st>>>(n, float(-a), s->nn_x.p, 1.0f, s->nn_res.p);
        *left = s->nn_res.p;
        s->nn_rejected_run = 0;
      } else {
        s->stats.learned_fallbacks++;
        s->nn_rejected_run++;
      }
      return SFX_OK;
    };
    auto cheb32 = [=](const float* b, float* z, cudaStream_t ss) -> int {
      return chebyshev<float, float>(s, apply_J32, s->diag32.p, s->lmax32, inner_degree(s), s->opt.chebyshev_ratio, b, z,
                                     s->cheb_d32.p, s->cheb_r32.p, ss);
    };
    if (o.mixed_precision) {
      // network step, then inner FP32 GMRES(k) + Jacobi-Chebyshev on what it leaves
      prec = [=](const double* v, double* z, cudaStream_t) -> int {
        sfx_blas::convert<double, float><<<nblocks(n), 256, 0, st>>>(n, v, s->b32.p);
        SFX_CUDA_TRY(cudaMemsetAsync(s->x32b.p, 0, sizeof(float) * n, st));
        const float* left = nullptr;
        if (int rc = nn_step(s->b32.p, s->x32b.p, &left)) return rc;
        // the captured inner cycle reads its right-hand side from b32
        if (left != s->b32.p)
          SFX_CUDA_TRY(cudaMemcpyAsync(s->b32.p, left, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
        if (int rc = inner_gmres(s, s->b32.p, s->x32.p, st)) return rc;
        sfx_blas::axpby<float><<<nblocks(n), 256, 0, st>>>(n, 1.0f, s->x32.p, 1.0f, s->x32b.p);
        sfx_blas::convert<float, double><<<nblocks(n), 256, 0, st>>>(n, s->x32b.p, z);
        return SFX_OK;
      };
    } else {
      // cycle 0: network, Chebyshev; cycle 1: Chebyshev, network, Chebyshev
      prec = [=](const double* v, double* z, cudaStream_t) -> int {
        sfx_blas::convert<double, float><<<nblocks(n), 256, 0, st>>>(n, v, s->b32.p);
        const float* res = s->b32.p;
        if (o.learned_cycle == 1) {
          if (int rc = cheb32(s->b32.p, s->x32b.p, st)) return rc;
          if (int rc = apply_J32(s, s->x32b.p, s->tmp32.p, st)) return rc;
          sfx_blas::rsub<float><<<nblocks(n), 256, 0, st>>>(n, s->b32.p, s->tmp32.p);
          res = s->tmp32.p;
        } else {
          SFX_CUDA_TRY(cudaMemsetAsync(s->x32b.p, 0, sizeof(float) * n, st));
        }
        const float* left = nullptr;
        if (int rc = nn_step(res, s->x32b.p, &left)) return rc;
        if (int rc = cheb32(left, s->x32.p, st)) return rc;
        sfx_blas::axpby<float><<<nblocks(n), 256, 0, st>>>(n, 1.0f, s->x32.p, 1.0f, s->x32b.p);
        sfx_blas::convert<float, double><<<nblocks(n), 256, 0, st>>>(n, s->x32b.p, z);
        return SFX_OK;
      };
    }
  } else if (o.mixed_precision) {
    // inner FP32 GMRES(k) with FP32 Jacobi-Chebyshev on the FP32 stored tangent
    const int k = o.inner_iterations;
    if (ensure(s->V32, size_t(k + 1) * n) || ensure(s->x32, n) || ensure(s->b32, n) || ensure(s->tmp32, n) ||
        ensure(s->diag32, n) || ensure(s->cheb_d32, n) || ensure(s->cheb_r32, n) || ensure(s->y32, size_t(k + 1)) ||
        ensure(s->tmp32b, n))
      return fail(SFX_ERR_NOMEM, "FP32 workspace allocation failed");
    sfx_blas::convert<double, float><<<nblocks(n), 256, 0, st>>>(n, s->diag.p, s->diag32.p);
    if (int rc = estimate_lmax<float, float>(s, apply_J32, s->diag32.p, s->tmp32.p, s->cheb_r32.p, s->cheb_d32.p,
                                             s->tmp32b.p, s->red32, &s->lmax32, st))
      return rc;
    prec = [=](const double* v, double* z, cudaStream_t) -> int {
      sfx_blas::convert<double, float><<<nblocks(n), 256, 0, st>>>(n, v, s->b32.p);
      if (int rc = inner_gmres(s, s->b32.p, s->x32.p, st)) return rc;
      sfx_blas::convert<float, double><<<nblocks(n), 256, 0, st>>>(n, s->x32.p, z);
      return SFX_OK;
    };
  } else {
    if (ensure(s->cheb_d, n) || ensure(s->cheb_r, n)) return fail(SFX_ERR_NOMEM, "workspace allocation failed");
    if (int rc = estimate_lmax<double, double>(s, apply_J64, s->diag.p, s->tmp.p, s->cheb_r.p, s->cheb_d.p, s->tmp2.p,
                                               s->red, &s->lmax, st))
      return rc;
    prec = [=](const double* v, double* z, cudaStream_t) -> int {
      return chebyshev<double, double>(s, apply_J64, s->diag.p, s->lmax, s->opt.chebyshev_degree,
                                       s->opt.chebyshev_ratio, v, z, s->cheb_d.p, s->cheb_r.p, st);
    };
  }
  SFX_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
  SFX_CUDA_TRY(cudaMemsetAsync(s->inner_count.p, 0, sizeof(int), st));
  s->nn_rejected_run = 0;
  const bool flexible = o.mixed_precision != 0 || o.krylov == SFX_KRYLOV_FGMRES || o.precond == SFX_PREC_LEARNED;
  int rc = gmres<double, double>(s, apply_J64, prec, flexible, rhs, x, s->V.p, s->Z.p, s->tmp.p, s->y.p, s->red, m,
                                 o.max_krylov_iterations, o.krylov_rel_tol, o.krylov_abs_tol, &iters, &rel, st);
  s->stats.krylov_iterations += iters;
  s->stats.last_krylov_rel = rel;
  if (rc == SFX_OK && o.mixed_precision) {
    int inner = 0;  // inner steps counted on the device by the captured cycles
    SFX_CUDA_TRY(cudaMemcpyAsync(&inner, s->inner_count.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SFX_CUDA_TRY(cudaStreamSynchronize(st));
    s->stats.inner_iterations += inner;
  }
  if (rc == SFX_OK && s->net && o.precond == SFX_PREC_LEARNED) {
    SFX_CUDA_TRY(cudaStreamSynchronize(st));
    if (int rw = check_waits(s->net)) return rw;
  }
  if (rc == SFX_OK && s->form->wait_error.raised()) {
    // a bounded wait inside a replayed FP32 action expired
    s->form->wait_error.clear();
    return fail(SFX_ERR_TIMEOUT, "a bulk-copy wait of the FP32 Jacobian action expired");
  }
  return rc;
}

}  // namespace

extern "C" {

int sfx_solver_default_options(sfx_solver_options* o) {
  if (!o) return fail(SFX_ERR_INVALID, "null options");
  *o = sfx_solver_options{};
  o->max_newton_iterations = 20;
  o->newton_rel_tol = 1e-8;
  o->newton_abs_tol = 1e-12;
  o->krylov = SFX_KRYLOV_GMRES;
  o->restart = 50;
  o->max_krylov_iterations = 300;
  o->krylov_rel_tol = 1e-8;
  o->krylov_abs_tol = 1e-12;
  o->precond = SFX_PREC_JACOBI_CHEBYSHEV;
  o->chebyshev_degree = 3;
  o->chebyshev_ratio = 30.0;
  o->eigen_iterations = 20;
  o->mixed_precision = 0;
  o->inner_iterations = 40;
  o->inner_rel_tol = 1e-3;
  o->print_level = 0;
  o->learned_cycle = 1;
  o->inner_chebyshev_degree = 0;
  o->learned_max_rejections = 3;
  return SFX_OK;
}

int sfx_solver_create(sfx_form form, const sfx_solver_options* opt, sfx_solver* out) {
  if (!form || !out) return fail(SFX_ERR_INVALID, "null argument");
  *out = nullptr;
  auto* s = new (std::nothrow) sfx_solver_s;
  if (!s) return fail(SFX_ERR_NOMEM, "host allocation failed");
  s->form = form;
  if (opt) s->opt = *opt;
  else sfx_solver_default_options(&s->opt);
  if (s->opt.restart < 1 || s->opt.chebyshev_degree < 1 || s->opt.inner_iterations < 1 ||
      s->opt.inner_iterations > 256 ||
      s->opt.inner_chebyshev_degree < 0 || s->opt.eigen_iterations < 2 || !(s->opt.chebyshev_ratio > 1.0) ||
      s->opt.learned_cycle < 0 || s->opt.learned_cycle > 1 || s->opt.learned_max_rejections < 0) {
    delete s;
    return fail(SFX_ERR_INVALID, "bad solver options");
  }
  sfx_form_num_dofs(form, &s->n);
  const size_t n = size_t(s->n);
  if (s->r.alloc(n) || s->du.alloc(n) || s->tmp.alloc(n) || s->tmp2.alloc(n) || s->diag.alloc(n) ||
      s->y.alloc(size_t(s->opt.restart + 1)) || s->V.alloc(4 * n) ||
      s->red.init(s->n, std::max(s->opt.restart, s->opt.inner_iterations) + 1) != cudaSuccess ||
      s->red32.init(s->n, s->opt.inner_iterations + 1) != cudaSuccess) {
    delete s;
    return fail(SFX_ERR_NOMEM, "solver workspace allocation failed");
  }
  if (cudaStreamCreateWithFlags(&s->capture, cudaStreamNonBlocking) != cudaSuccess) {
    delete s;
    return fail(SFX_ERR_CUDA, "capture stream creation failed");
  }
  if (s->gstate.alloc(size_t(sfx_blas::GmresLayout{s->opt.inner_iterations}.size())) != cudaSuccess ||
      s->inner_count.alloc(1) != cudaSuccess || cudaMemset(s->inner_count.p, 0, sizeof(int)) != cudaSuccess) {
    delete s;
    return fail(SFX_ERR_NOMEM, "solver workspace allocation failed");
  }
  *out = s;
  return SFX_OK;
}

int sfx_solver_destroy(sfx_solver s) {
  delete s;
  return SFX_OK;
}

int sfx_solver_set_essential(sfx_solver s, const int64_t* dofs, int64_t n) {
  if (!s || (n > 0 && !dofs)) return fail(SFX_ERR_INVALID, "null argument");
  for (int64_t i = 0; i < n; i++)
    if (dofs[i] < 0 || dofs[i] >= s->n) return fail(SFX_ERR_INVALID, "essential dof out of range");
  s->n_ess = n;
  if (n == 0) return SFX_OK;
  if (s->ess.upload(dofs, size_t(n)) != cudaSuccess) return fail(SFX_ERR_CUDA, "upload essential dofs");
  return SFX_OK;
}

int sfx_solver_solve_linear(sfx_solver s, double t, const double* u_lin, const double* rhs, double* x, void* stream) {
  if (!s || !u_lin || !rhs || !x) return fail(SFX_ERR_INVALID, "null argument");
  auto st = static_cast<cudaStream_t>(stream);
  s->stats = sfx_solver_stats{};
  if (int rc = sfx_linearize(s->form, t, u_lin, nullptr, st)) return rc;
  SFX_CUDA_TRY(cudaMemcpyAsync(s->r.p, rhs, sizeof(double) * size_t(s->n), cudaMemcpyDeviceToDevice, st));
  if (s->n_ess) sfx_blas::set_entries<double><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 0.0, s->r.p);
  return linear_solve(s, s->r.p, x, st);
}

int sfx_solver_solve_adjoint(sfx_solver s, double t, const double* u_lin, const double* rhs, double* x,
                             void* stream) {
  if (!s || !u_lin || !rhs || !x) return fail(SFX_ERR_INVALID, "null argument");
  auto st = static_cast<cudaStream_t>(stream);
  s->stats = sfx_solver_stats{};
  if (int rc = sfx_linearize(s->form, t, u_lin, nullptr, st)) return rc;
  SFX_CUDA_TRY(cudaMemcpyAsync(s->r.p, rhs, sizeof(double) * size_t(s->n), cudaMemcpyDeviceToDevice, st));
  if (s->n_ess) sfx_blas::set_entries<double><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 0.0, s->r.p);
  s->transpose = true;
  const int rc = linear_solve(s, s->r.p, x, st);
  s->transpose = false;
  s->drop_graphs();  // the captured inner cycle applies J^T
  return rc;
}

int sfx_solver_solve(sfx_solver s, double t, double* u, void* stream) {
  if (!s || !u) return fail(SFX_ERR_INVALID, "null argument");
  auto st = static_cast<cudaStream_t>(stream);
  const int64_t n = s->n;
  s->stats = sfx_solver_stats{};
  cudaError_t err;
  // r = R(u), zero on the essential set
  if (int rc = sfx_residual(s->form, t, u, s->r.p, st)) return rc;
  if (s->n_ess) sfx_blas::set_entries<double><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 0.0, s->r.p);
  double r0 = std::sqrt(s->red.dot(s->r.p, s->r.p, n, st, &err));
  SFX_CUDA_TRY(err);
  if (!std::isfinite(r0)) return fail(SFX_ERR_NONFINITE, "non-finite initial residual");
  s->stats.initial_residual = r0;
  double rn = r0;
  const double target = std::max(s->opt.newton_rel_tol * r0, s->opt.newton_abs_tol);
  int it = 0;
  for (it = 0; it < s->opt.max_newton_iterations && rn > target; it++) {
    if (int rc = sfx_linearize(s->form, t, u, nullptr, st)) return rc;
    if (int rc = linear_solve(s, s->r.p, s->du.p, st)) return rc;
    sfx_blas::axpby<double><<<nblocks(n), 256, 0, st>>>(n, -1.0, s->du.p, 1.0, u);
    if (int rc = sfx_residual(s->form, t, u, s->r.p, st)) return rc;
    if (s->n_ess) sfx_blas::set_entries<double><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 0.0, s->r.p);
    rn = std::sqrt(s->red.dot(s->r.p, s->r.p, n, st, &err));
    SFX_CUDA_TRY(err);
    if (!std::isfinite(rn)) return fail(SFX_ERR_NONFINITE, "non-finite residual in Newton");
    if (s->opt.print_level > 0)
      std::fprintf(stderr, "newton %d  |r| = %.6e  rel = %.3e  krylov %d\n", it + 1, rn, rn / (r0 > 0 ? r0 : 1.0),
                   s->stats.krylov_iterations);
  }
  s->stats.newton_iterations = it;
  s->stats.final_residual = rn;
  s->stats.converged = rn <= target ? 1 : 0;
  return s->stats.converged ? SFX_OK : fail(SFX_ERR_NOT_CONVERGED, "Newton did not converge");
}

int sfx_solver_warm_start(sfx_solver s, double t, double* u, const double* u_target, void* stream) {
  if (!s || !u || !u_target) return fail(SFX_ERR_INVALID, "null argument");
  auto st = static_cast<cudaStream_t>(stream);
  const int64_t n = s->n;
  s->stats = sfx_solver_stats{};
  if (s->n_ess == 0) return SFX_OK;
  if (ensure(s->wx, size_t(n))) return fail(SFX_ERR_NOMEM, "workspace allocation failed");
  // d: the essential-value increment, zero elsewhere
  SFX_CUDA_TRY(cudaMemsetAsync(s->du.p, 0, sizeof(double) * n, st));
  sfx_blas::diff_entries<double><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, u_target, u, s->du.p);
  // rhs = -J(u) d on the free rows, 0 on the essential rows
  if (int rc = sfx_linearize(s->form, t, u, nullptr, st)) return rc;
  if (int rc = sfx_jvp(s->form, s->du.p, s->r.p, st)) return rc;
  sfx_blas::scale<double><<<nblocks(n), 256, 0, st>>>(n, -1.0, s->r.p);
  sfx_blas::set_entries<double><<<nblocks(s->n_ess), 256, 0, st>>>(s->n_ess, s->ess.p, 0.0, s->r.p);
  // x = J_ff^-1 rhs (x = 0 on the essential rows); u += d + x
  if (int rc = linear_solve(s, s->r.p, s->wx.p, st)) return rc;
  sfx_blas::axpby<double><<<nblocks(n), 256, 0, st>>>(n, 1.0, s->du.p, 1.0, u);
  sfx_blas::axpby<double><<<nblocks(n), 256, 0, st>>>(n, 1.0, s->wx.p, 1.0, u);
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

int sfx_solver_set_learned(sfx_solver s, sfx_lnet net, int nx, int ny, int nz, const float* features) {
  if (!s || !net || !features) return fail(SFX_ERR_INVALID, "null argument");
  if (s->form->general) return fail(SFX_ERR_UNSUPPORTED, "the learned preconditioner needs a structured node grid");
  if (int64_t(nx) * ny * nz * 3 != s->n) return fail(SFX_ERR_INVALID, "node grid does not match the form (3 components)");
  s->net = net;
  s->grid[0] = nx;
  s->grid[1] = ny;
  s->grid[2] = nz;
  s->features = features;
  return SFX_OK;
}

int sfx_solver_get_stats(sfx_solver s, sfx_solver_stats* out) {
  if (!s || !out) return fail(SFX_ERR_INVALID, "null argument");
  *out = s->stats;
  return SFX_OK;
}

}  // extern "C"
