// sfx — quantities of interest: Functional<double(H1<p,c>)>
// (functional_qoi.inl:58-528, finite_element<g, QOI> in detail/qoi.inl).
//
// A QoI integrates a scalar q-function over the domain and / or boundary
// faces: Q(u) = sum_e sum_q q(t, X, u, grad u) det(J) w  (+ faces, weighted
// by |dX/ds x dX/dt| w).  Three evaluations share the element layout of the
// residual kernels (one warp per Q2 element, four Q1 elements per warp):
//   QOI_VALUE     per-element sums of q det(J) w
//   QOI_ACTION    per-element sums of dq(du) det(J) w (directional duals) —
//                 serac's Gradient::operator()(dx), functional_qoi.inl:420
//   QOI_GRADIENT  dQ/du as an E-vector: dq/du and dq/d(grad u) at each point
//                 (one directional dual per input), integrated against the
//                 basis like a residual's source and flux — serac's
//                 Gradient::assemble(), functional_qoi.inl:422-475 — plus the
//                 per-element values
// Per-element (per-face) values are summed along the lanes in a fixed order,
// then reduced on the device by a two-pass fixed-shape tree (qoi_sum):
// deterministic.
#pragma once

#include "sfx/boundary.cuh"
#include "sfx/kernels.cuh"

namespace sfx {

/// Built-in QoI integrands of the C ABI.  Domain ones are called as
/// q(t, tuple{X, dX/dxi}, tuple{u, du/dX}), face ones as
/// q(t, tuple{X, dX/d(s,t)}, tuple{u, du/d(s,t)}); both return a scalar.
namespace qoi_models {

struct Measure {
  template <typename Pos, typename Arg>
  SFX_HDI double operator()(double, const Pos&, const Arg&) const {
    return 1.0;
  }
};

/// a . X (first moments of the region)
struct PositionMoment {
  double a[3];
  template <typename Pos, typename Arg>
  SFX_HDI auto operator()(double, const Pos& pos, const Arg&) const {
    const auto& X = get<0>(pos);
    return a[0] * X[0] + a[1] * X[1] + a[2] * X[2];
  }
};

template <int C, typename V>
SFX_HDI auto component(const V& v, int c) {
  if constexpr (C == 1) {
    (void)c;
    return v;
  } else {
    return v[c];
  }
}

/// w . u (weighted field integral; averages, reaction-free displacement measures)
template <int C>
struct FieldIntegral {
  double w[C];
  template <typename Pos, typename Arg>
  SFX_HDI auto operator()(double, const Pos&, const Arg& arg) const {
    const auto& u = get<0>(arg);
    auto s = w[0] * component<C>(u, 0);
#pragma unroll
    for (int c = 1; c < C; c++) s = s + w[c] * component<C>(u, c);
    return s;
  }
};

/// Stored energy of the Neo-Hookean model of SFX_MAT_NEOHOOKEAN
/// (solid_material.hpp:98-127): with H = du/dX, J = det(I + H),
///   W = G/2 (|H|^2 + 2 tr H) - G ln J + lambda/2 (ln J)^2,  lambda = K - 2G/3,
/// whose derivative dW/dH is that model's first Piola stress
/// lambda ln J F^-T + G (F - F^-T), so dQ/du equals the model's residual.
struct NeoHookeanEnergy {
  double K, G;
  template <typename Pos, typename Arg>
  SFX_HDI auto operator()(double, const Pos&, const Arg& arg) const {
    using std::log1p;
    const auto& H = get<1>(arg);
    const double lambda = K - (2.0 / 3.0) * G;
    const auto lnJ = log1p(detApIm1(H));
    // |H|^2 + 2 tr H = tr(F^T F) - 3, formed without the cancellation of the latter
    auto h2 = H[0][0] * (H[0][0] + 2.0);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        if (i + j > 0) h2 = h2 + H[i][j] * H[i][j];
    h2 = h2 + 2.0 * (H[1][1] + H[2][2]);
    return 0.5 * G * h2 - G * lnJ + 0.5 * lambda * lnJ * lnJ;
  }
};

/// u . n on faces (c = 3), n the unit outward normal: the first-order change
/// of the enclosed volume under the displacement u
struct NormalField {
  template <typename Pos, typename Arg>
  SFX_HDI auto operator()(double, const Pos& pos, const Arg& arg) const {
    using std::sqrt;
    const auto& J = get<1>(pos);
    const auto& u = get<0>(arg);
    const auto n0 = J[1][0] * J[2][1] - J[2][0] * J[1][1];
    const auto n1 = J[2][0] * J[0][1] - J[0][0] * J[2][1];
    const auto n2 = J[0][0] * J[1][1] - J[1][0] * J[0][1];
    const auto inv = 1.0 / sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    return (n0 * inv) * u[0] + (n1 * inv) * u[1] + (n2 * inv) * u[2];
  }
};

/// Nonlinear test integrand with value, gradient and position dependence
/// (domain): X0^2 + sin X1 + X0 s^3 + (1 + X2)/2 |grad u|^2, s = sum_c u_c
template <int C>
struct PolyTest {
  template <typename Pos, typename Arg>
  SFX_HDI auto operator()(double, const Pos& pos, const Arg& arg) const {
    using std::sin;
    const auto& X = get<0>(pos);
    const auto& u = get<0>(arg);
    const auto& g = get<1>(arg);
    auto s = component<C>(u, 0);
#pragma unroll
    for (int c = 1; c < C; c++) s = s + component<C>(u, c);
    auto g2 = component<C>(g, 0)[0] * component<C>(g, 0)[0];
#pragma unroll
    for (int c = 0; c < C; c++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        if (c + j > 0) g2 = g2 + component<C>(g, c)[j] * component<C>(g, c)[j];
    return X[0] * X[0] + sin(X[1]) + X[0] * s * s * s + 0.5 * (1.0 + X[2]) * g2;
  }
};

/// Nonlinear test integrand on faces: X0 - X1 + cos(s X1) + |du/ds|^2 / 4
template <int C>
struct PolyTestFace {
  template <typename Pos, typename Arg>
  SFX_HDI auto operator()(double, const Pos& pos, const Arg& arg) const {
    using std::cos;
    const auto& X = get<0>(pos);
    const auto& u = get<0>(arg);
    const auto& g = get<1>(arg);
    auto s = component<C>(u, 0);
#pragma unroll
    for (int c = 1; c < C; c++) s = s + component<C>(u, c);
    auto gs = component<C>(g, 0)[0] * component<C>(g, 0)[0];
#pragma unroll
    for (int c = 1; c < C; c++) gs = gs + component<C>(g, c)[0] * component<C>(g, c)[0];
    return X[0] - X[1] + cos(s * X[1]) + 0.25 * gs;
  }
};

}  // namespace qoi_models

namespace kernels {

enum { QOI_VALUE = 0, QOI_ACTION = 1, QOI_GRADIENT = 2 };

/// Sum of v over the NQ lanes [base, base + NQ) in lane order; every lane of
/// the segment gets the same result.
template <int NQ, typename Real>
SFX_HDI Real segment_sum(Real v, int base) {
  Real acc = 0;
#pragma unroll
  for (int k = 0; k < NQ; k++) acc += shfl(v, base + k);
  return acc;
}

/// Domain QoI over all elements.  elem_val[e] receives the element's value
/// (QOI_VALUE, QOI_GRADIENT) or directional derivative (QOI_ACTION; a.du is
/// the direction); QOI_GRADIENT also writes dQ/du into a.out_e [e][c][node].
template <int P, int C, int MODE, typename QF>
__global__ void __launch_bounds__(128) qoi_domain_kernel(DomainArgs<double> a, QF qf, double* __restrict__ elem_val) {
  using Real = double;
  using S = dual<Real, Real>;
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q * Q;
  constexpr int EPW = 32 / NQ;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / NQ;
  const int qi_raw = lane - sub * NQ;
  const bool slot = sub < EPW;
  const int qi = slot ? qi_raw : NQ - 1;
  const int base = slot ? sub * NQ : 0;
  const int64_t e = warp * EPW + (slot ? sub : 0);
  const bool valid = slot && e < a.num_elements;
  const int ix = qi % Q, iy = (qi / Q) % Q, iz = qi / (Q * Q);

  __shared__ Real sB[Q][Q], sG[Q][Q];
  if (threadIdx.x < Q * Q) {
    int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = basis_table<P>().B[i][j];
    sG[i][j] = basis_table<P>().G[i][j];
  }
  __syncthreads();

  const int64_t nq_total = a.num_elements * NQ;
  const int64_t gq = e * NQ + qi;
  const int32_t node = valid ? a.conn[e * NQ + qi] : 0;

  Real uv[C], ug[C][3], dv[C], dg[C][3];
#pragma unroll
  for (int c = 0; c < C; c++) {
    const Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    interpolate_lane<Q, Real>(U, base, ix, iy, iz, sB, sG, uv[c], ug[c][0], ug[c][1], ug[c][2]);
    if constexpr (MODE == QOI_ACTION) {
      const Real dU = valid ? a.du[c * a.num_nodes + node] : Real(0);
      interpolate_lane<Q, Real>(dU, base, ix, iy, iz, sB, sG, dv[c], dg[c][0], dg[c][1], dg[c][2]);
    }
  }
  Real Ji[3][3];
  Real dvol = 0;
  tensor<Real, 3> X{};
  tensor<Real, 3, 3> Jm{};
  if (valid) {
    const Real* g = a.geom + gq;
#pragma unroll
    for (int k = 0; k < 9; k++) Ji[k / 3][k % 3] = g[k * nq_total];
    dvol = g[9 * nq_total];
#pragma unroll
    for (int k = 0; k < 3; k++) X[k] = g[(10 + k) * nq_total];
#pragma unroll
    for (int k = 0; k < 9; k++) Jm[k / 3][k % 3] = g[(13 + k) * nq_total];
  } else {
#pragma unroll
    for (int k = 0; k < 9; k++) Ji[k / 3][k % 3] = Real(k % 4 == 0);
  }
  const auto position = tuple{X, Jm};
  // physical gradients (finite_element.hpp:246-273)
  Real gx[C][3], dgx[C][3];
#pragma unroll
  for (int c = 0; c < C; c++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      gx[c][j] = ug[c][0] * Ji[0][j] + ug[c][1] * Ji[1][j] + ug[c][2] * Ji[2][j];
      if constexpr (MODE == QOI_ACTION) dgx[c][j] = dg[c][0] * Ji[0][j] + dg[c][1] * Ji[1][j] + dg[c][2] * Ji[2][j];
    }

  Real point = 0;  // this point's contribution to the element sum
  if constexpr (MODE == QOI_VALUE) {
    value_t<C, Real> qv{};
    grad_t<C, Real> qg{};
#pragma unroll
    for (int c = 0; c < C; c++) {
      comp<C>(qv, c) = uv[c];
#pragma unroll
      for (int j = 0; j < 3; j++) comp<C>(qg, c)[j] = gx[c][j];
    }
    point = dvol * Real(get_value(qf(a.t, position, tuple{qv, qg})));
  } else if constexpr (MODE == QOI_ACTION) {
    value_t<C, S> qv{};
    grad_t<C, S> qg{};
#pragma unroll
    for (int c = 0; c < C; c++) {
      comp<C>(qv, c) = S{uv[c], dv[c]};
#pragma unroll
      for (int j = 0; j < 3; j++) comp<C>(qg, c)[j] = S{gx[c][j], dgx[c][j]};
    }
    point = dvol * part<JVP, Real>(qf(a.t, position, tuple{qv, qg}));
  } else {
    // one directional dual per input: value of component k (k < C), then the
    // parent-space gradient entry (c, b) of k = C + 3c + b
    Real src[C] = {}, flx[C][3] = {};
#pragma unroll 1
    for (int k = 0; k < 4 * C; k++) {
      const int seed_c = k < C ? k : (k - C) / 3;
      const int seed_b = k < C ? -1 : (k - C) % 3;
      value_t<C, S> qv{};
      grad_t<C, S> qg{};
#pragma unroll
      for (int c = 0; c < C; c++) {
        comp<C>(qv, c) = S{uv[c], Real(c == seed_c && seed_b < 0)};
#pragma unroll
        for (int j = 0; j < 3; j++)
          comp<C>(qg, c)[j] = S{gx[c][j], (c == seed_c && seed_b >= 0) ? Ji[seed_b][j] : Real(0)};
      }
      const auto out = qf(a.t, position, tuple{qv, qg});
      const Real d = dvol * part<JVP, Real>(out);
      if (k == 0) point = dvol * Real(get_value(out));
#pragma unroll
      for (int c = 0; c < C; c++) {
        if (k == c) src[c] = d;
#pragma unroll
        for (int b = 0; b < 3; b++)
          if (k == C + 3 * c + b) flx[c][b] = d;
      }
    }
#pragma unroll
    for (int c = 0; c < C; c++) {
      const Real r = integrate_lane<Q, true, true, Real>(src[c], flx[c][0], flx[c][1], flx[c][2], base, ix, iy, iz,
                                                         sB, sG);
      if (valid) a.out_e[(e * C + c) * NQ + qi] = r;
    }
  }
  const Real total = segment_sum<NQ, Real>(valid ? point : Real(0), base);
  if (valid && qi_raw == 0) elem_val[e] = total;
}

/// Face QoI over the faces of one face set (same modes as qoi_domain_kernel;
/// face_val[f] per face, QOI_GRADIENT writes dQ/du into a.out_e [f][c][node]).
template <int P, int C, int MODE, typename QF>
__global__ void __launch_bounds__(128) qoi_face_kernel(FaceArgs<double> a, QF qf, double* __restrict__ face_val) {
  using Real = double;
  using S = dual<Real, Real>;
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q;
  constexpr int FPW = 32 / NQ;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / NQ;
  const int qi_raw = lane - sub * NQ;
  const bool slot = sub < FPW;
  const int qi = slot ? qi_raw : NQ - 1;
  const int base = slot ? sub * NQ : 0;
  const int64_t f = warp * FPW + (slot ? sub : 0);
  const bool valid = slot && f < a.num_faces;
  const int ix = qi % Q, iy = qi / Q;

  __shared__ Real sB[Q][Q], sG[Q][Q];
  if (threadIdx.x < Q * Q) {
    int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = basis_table<P>().B[i][j];
    sG[i][j] = basis_table<P>().G[i][j];
  }
  __syncthreads();
  const int64_t nq_total = a.num_faces * NQ;
  const int64_t gq = f * NQ + qi;
  const int32_t node = valid ? a.fconn[f * NQ + qi] : 0;

  Real uv[C], us[C], ut[C], dv[C], ds[C], dt[C];
#pragma unroll
  for (int c = 0; c < C; c++) {
    const Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    face_interpolate<Q, Real>(U, base, ix, iy, sB, sG, uv[c], us[c], ut[c]);
    if constexpr (MODE == QOI_ACTION) {
      const Real dU = valid ? a.du[c * a.num_nodes + node] : Real(0);
      face_interpolate<Q, Real>(dU, base, ix, iy, sB, sG, dv[c], ds[c], dt[c]);
    }
  }
  tensor<double, 3> X{};
  tensor<double, 3, 2> J{};
  Real scale = 0;
  if (valid) {
    const double* g = a.fgeom + gq;
#pragma unroll
    for (int k = 0; k < 3; k++) X[k] = g[k * nq_total];
#pragma unroll
    for (int k = 0; k < 6; k++) J[k / 2][k % 2] = g[(3 + k) * nq_total];
    scale = g[9 * nq_total];
  } else {
    // a non-degenerate frame for idle lanes (their results are discarded)
    J[0][0] = 1.0;
    J[1][1] = 1.0;
  }
  const auto position = tuple{X, J};

  Real point = 0;
  if constexpr (MODE == QOI_VALUE) {
    fvalue_t<C, Real> qv{};
    fgrad_t<C, Real> qg{};
#pragma unroll
    for (int c = 0; c < C; c++) {
      comp<C>(qv, c) = uv[c];
      comp<C>(qg, c)[0] = us[c];
      comp<C>(qg, c)[1] = ut[c];
    }
    point = scale * Real(get_value(qf(a.t, position, tuple{qv, qg})));
  } else if constexpr (MODE == QOI_ACTION) {
    fvalue_t<C, S> qv{};
    fgrad_t<C, S> qg{};
#pragma unroll
    for (int c = 0; c < C; c++) {
      comp<C>(qv, c) = S{uv[c], dv[c]};
      comp<C>(qg, c)[0] = S{us[c], ds[c]};
      comp<C>(qg, c)[1] = S{ut[c], dt[c]};
    }
    point = scale * part<JVP, Real>(qf(a.t, position, tuple{qv, qg}));
  } else {
#pragma unroll 1
    for (int cj = 0; cj < C; cj++) {
      Real w[3];
#pragma unroll
      for (int b = 0; b < 3; b++) {
        fvalue_t<C, S> qv{};
        fgrad_t<C, S> qg{};
#pragma unroll
        for (int c = 0; c < C; c++) {
          comp<C>(qv, c) = S{uv[c], Real(c == cj && b == 0)};
          comp<C>(qg, c)[0] = S{us[c], Real(c == cj && b == 1)};
          comp<C>(qg, c)[1] = S{ut[c], Real(c == cj && b == 2)};
        }
        const auto out = qf(a.t, position, tuple{qv, qg});
        w[b] = scale * part<JVP, Real>(out);
        if (cj == 0 && b == 0) point = scale * Real(get_value(out));
      }
      const Real r = face_integrate_full<Q, Real>(w[0], w[1], w[2], base, ix, iy, sB, sG);
      if (valid) a.out_e[(f * C + cj) * NQ + qi] = r;
    }
  }
  const Real total = segment_sum<NQ, Real>(valid ? point : Real(0), base);
  if (valid && qi_raw == 0) face_val[f] = total;
}

/// Deterministic sum of x[0, n): block b sums its fixed chunk with a fixed
/// tree into partial[b]; qoi_sum_final adds the partials in order.
constexpr int kQoiSumBlock = 256;
constexpr int kQoiMaxPartials = 512;


template <typename T>
__global__ void __launch_bounds__(kQoiSumBlock) qoi_sum_partial(const T* __restrict__ x, int64_t n,
                                                                T* __restrict__ partial) {
  __shared__ T sh[kQoiSumBlock];
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = int64_t(blockIdx.x) * chunk;
  const int64_t b1 = b0 + chunk < n ? b0 + chunk : n;
  T acc = 0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += kQoiSumBlock) acc += x[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kQoiSumBlock / 2; s > 0; s >>= 1) {
    if (int(threadIdx.x) < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

/// out[0] = sum of the nb partials (one block), fixed order
template <typename T>
__global__ void __launch_bounds__(kQoiSumBlock) qoi_sum_final(const T* __restrict__ partial, int nb,
                                                              T* __restrict__ out) {
  __shared__ T sh[kQoiSumBlock];
  T acc = 0;
  for (int i = threadIdx.x; i < nb; i += kQoiSumBlock) acc += partial[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kQoiSumBlock / 2; s > 0; s >>= 1) {
    if (int(threadIdx.x) < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

/// Launches the two-pass sum of x[0, n) into out[0] (partial: kQoiMaxPartials entries).
inline cudaError_t qoi_sum(const double* x, int64_t n, double* partial, double* out, cudaStream_t s) {
  const int64_t want = (n + kQoiSumBlock - 1) / kQoiSumBlock;
  const int nb = int(want < kQoiMaxPartials ? (want > 0 ? want : 1) : kQoiMaxPartials);
  qoi_sum_partial<double><<<nb, kQoiSumBlock, 0, s>>>(x, n, partial);
  qoi_sum_final<double><<<1, kQoiSumBlock, 0, s>>>(partial, nb, out);
  return cudaGetLastError();
}

}  // namespace kernels
}  // namespace sfx
