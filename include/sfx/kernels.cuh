// sfx — fused element kernels for H1 hexahedra on sm_103a.
//
// One warp owns the quadrature points of one Q2 element (27 of 32 lanes) or
// of four Q1 elements (8 lanes each).  Lane i holds quadrature point i and,
// before interpolation / after integration, element node i (n = q = p + 1).
// The sum-factorised tensor contractions of serac's hexahedron_H1.inl:169-280
// are carried out with warp shuffles (no shared memory, no barriers):
//   interpolate: x-pass, y-pass, z-pass produce u and grad_xi u at each point
//   q-function : in registers, with forward-mode duals for the tangent
//   integrate  : transposed passes; each lane ends with one nodal residual
// Element residuals go to an E-vector; a node-owner kernel sums them into the
// global vector in a fixed order (no floating-point atomics: deterministic).
#pragma once

#include <cuda_fp16.h>

#include <cstdint>
#include <type_traits>
#include <utility>

#include "sfx/dual.hpp"
#include "sfx/materials.hpp"
#include "sfx/bulk.cuh"
#include "sfx/quadrature.hpp"
#include "sfx/tensor.hpp"
#include "sfx/tuple.hpp"

namespace sfx {
namespace kernels {

enum Mode : int { RESIDUAL = 0, RESIDUAL_UPDATE = 1, JVP = 2 };

/// Geometric factors per quadrature point, structure-of-arrays over all points
/// of the mesh (index k * nq_total + e * nq + q):
///   k = 0..8   J^{-1}  (row-major, [xi][x])
///   k = 9      det(J) * w_q
///   k = 10..12 X (position)
///   k = 13..21 J = dX/dxi (row-major, [x][xi])
constexpr int GEOM_STRIDE = 22;

template <typename Real>
struct DomainArgs {
  const Real* u;          // L-vector (byNODES) of the trial field
  const Real* du;         // direction for JVP
  Real* out_e;            // E-vector [e][c][node]
  const int32_t* conn;    // [e][node] global node ids
  const Real* geom;       // GEOM_STRIDE x nq_total
  double* state;          // quadrature-point state, SoA [k][e*nq+q] (doubles)
  const double* params;   // per-element material parameters [e][nparams]
  int64_t num_nodes;
  int64_t num_elements;
  double t;
};

template <int C, typename T>
using value_t = std::conditional_t<C == 1, T, tensor<T, C>>;
template <int C, typename T>
using grad_t = std::conditional_t<C == 1, tensor<T, 3>, tensor<T, C, 3>>;

template <int C, typename V>
SFX_HDI auto& comp(V& v, int c) {
  if constexpr (C == 1) {
    (void)c;
    return v;
  } else {
    return v[c];
  }
}

// component c of a q-function source output (zero / scalar / vector)
template <int C, typename S>
SFX_HDI auto source_comp(const S& s, int c) {
  if constexpr (is_zero<S>::value) {
    (void)c;
    return zero{};
  } else if constexpr (C == 1 && !is_tensor<S>::value) {
    (void)c;
    return s;
  } else {
    return s[c];
  }
}
// row c of a q-function flux output (zero / tensor<3> / tensor<C,3>)
template <int C, typename F>
SFX_HDI auto flux_row(const F& f, int c) {
  if constexpr (is_zero<F>::value) {
    (void)c;
    return zero{};
  } else if constexpr (C == 1 && F::ndim == 1) {
    (void)c;
    return f;
  } else {
    return f[c];
  }
}

template <typename T>
struct base_scalar {
  using type = T;
};
template <typename T, int... n>
struct base_scalar<tensor<T, n...>> {
  using type = typename base_scalar<T>::type;
};

// whether the requested part (value for residual, directional derivative for
// JVP) of a q-function output is structurally nonzero
template <int MODE, typename T>
constexpr bool has_part() {
  using B = typename base_scalar<T>::type;
  if constexpr (is_zero<B>::value) return false;
  else if constexpr (MODE == JVP) return is_dual<B>::value;
  else return true;
}

template <int MODE, typename Real, typename T>
SFX_HDI Real part(const T& x) {
  if constexpr (MODE == JVP) {
    if constexpr (is_dual<T>::value) return Real(x.gradient);
    else return Real(0);
  } else {
    return Real(get_value(x));
  }
}

template <typename Real>
SFX_HDI Real shfl(Real v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

/// Interpolate one nodal field held one node per lane into the value and the
/// three parent-space derivatives at this lane's quadrature point.
template <int Q, typename Real>
SFX_HDI void interpolate_lane(Real U, int base, int ix, int iy, int iz, const Real (*B)[Q], const Real (*G)[Q],
                              Real& val, Real& g0, Real& g1, Real& g2) {
  // x-pass: A0(qx, ny, nz), A1(qx, ny, nz)
  Real A0 = 0, A1 = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    Real v = shfl(U, base + k + Q * (iy + Q * iz));
    A0 += B[ix][k] * v;
    A1 += G[ix][k] * v;
  }
  // y-pass: C00 (B_y B_x), C10 (B_y G_x), C01 (G_y B_x)
  Real C00 = 0, C10 = 0, C01 = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    int src = base + ix + Q * (k + Q * iz);
    Real a0 = shfl(A0, src);
    Real a1 = shfl(A1, src);
    C00 += B[iy][k] * a0;
    C10 += B[iy][k] * a1;
    C01 += G[iy][k] * a0;
  }
  // z-pass
  Real v = 0, gx = 0, gy = 0, gz = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    int src = base + ix + Q * (iy + Q * k);
    Real c00 = shfl(C00, src);
    Real c10 = shfl(C10, src);
    Real c01 = shfl(C01, src);
    v += B[iz][k] * c00;
    gx += B[iz][k] * c10;
    gy += B[iz][k] * c01;
    gz += G[iz][k] * c00;
  }
  val = v;
  g0 = gx;
  g1 = gy;
  g2 = gz;
}

/// Integrate (s, f) given at this lane's quadrature point against the basis,
/// returning the nodal residual of this lane's node.  HS / HF drop the source
/// / flux terms when they are structurally zero.
template <int Q, bool HS, bool HF, typename Real>
SFX_HDI Real integrate_lane(Real s, Real f0, Real f1, Real f2, int base, int ix, int iy, int iz, const Real (*B)[Q],
                            const Real (*G)[Q]) {
  // x-pass over qx: a = sum B[q][nx] s + G[q][nx] f0, b = sum B f1, c = sum B f2
  Real a = 0, b = 0, c = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    int src = base + k + Q * (iy + Q * iz);
    if constexpr (HS) a += B[k][ix] * shfl(s, src);
    if constexpr (HF) {
      a += G[k][ix] * shfl(f0, src);
      b += B[k][ix] * shfl(f1, src);
      c += B[k][ix] * shfl(f2, src);
    }
  }
  // y-pass: d = sum B[q][ny] a + G[q][ny] b ; e = sum B[q][ny] c
  Real d = 0, e = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    int src = base + ix + Q * (k + Q * iz);
    d += B[k][iy] * shfl(a, src);
    if constexpr (HF) {
      d += G[k][iy] * shfl(b, src);
      e += B[k][iy] * shfl(c, src);
    }
  }
  // z-pass: r = sum B[q][nz] d + G[q][nz] e
  Real r = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    int src = base + ix + Q * (iy + Q * k);
    r += B[k][iz] * shfl(d, src);
    if constexpr (HF) r += G[k][iz] * shfl(e, src);
  }
  return r;
}

/// interpolate_lane by collocation: the nodal field is first interpolated to
/// the quadrature points (B along x, y, z: 3Q multiply-adds), then the point
/// values are differentiated with the collocated derivative matrix Dq = G B^-1
/// (3Q more).  Same result as interpolate_lane to rounding with 6Q instead of
/// 8Q (gradient only) or 9Q (value and gradient) multiply-adds per lane — the
/// cost that bounds the FP64 Jacobian action.
template <int Q, typename Real>
SFX_HDI void interpolate_colloc(Real U, int base, int ix, int iy, int iz, const Real (*B)[Q], const Real (*Dq)[Q],
                                Real& val, Real& g0, Real& g1, Real& g2) {
  Real a = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) a += B[ix][k] * shfl(U, base + k + Q * (iy + Q * iz));
  Real b = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) b += B[iy][k] * shfl(a, base + ix + Q * (k + Q * iz));
  Real w = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) w += B[iz][k] * shfl(b, base + ix + Q * (iy + Q * k));
  Real d0 = 0, d1 = 0, d2 = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    d0 += Dq[ix][k] * shfl(w, base + k + Q * (iy + Q * iz));
    d1 += Dq[iy][k] * shfl(w, base + ix + Q * (k + Q * iz));
    d2 += Dq[iz][k] * shfl(w, base + ix + Q * (iy + Q * k));
  }
  val = w;
  g0 = d0;
  g1 = d1;
  g2 = d2;
}

/// integrate_lane by collocation, the transpose of interpolate_colloc: the
/// flux is taken back through Dq^T at the points and added to the source,
/// then B^T is applied along x, y, z.
template <int Q, bool HS, bool HF, typename Real>
SFX_HDI Real integrate_colloc(Real s, Real f0, Real f1, Real f2, int base, int ix, int iy, int iz, const Real (*B)[Q],
                              const Real (*Dq)[Q]) {
  Real t = HS ? s : Real(0);
#pragma unroll
  for (int k = 0; k < (HF ? Q : 0); k++) {
    t += Dq[k][ix] * shfl(f0, base + k + Q * (iy + Q * iz));
    t += Dq[k][iy] * shfl(f1, base + ix + Q * (k + Q * iz));
    t += Dq[k][iz] * shfl(f2, base + ix + Q * (iy + Q * k));
  }
  Real a = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) a += B[k][ix] * shfl(t, base + k + Q * (iy + Q * iz));
  Real b = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) b += B[k][iy] * shfl(a, base + ix + Q * (k + Q * iz));
  Real r = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) r += B[k][iz] * shfl(b, base + ix + Q * (iy + Q * k));
  return r;
}

template <typename State>
SFX_HDI void load_state(State& s, const double* state, int64_t gq, int64_t nq_total) {
  constexpr int n = sizeof(State) / sizeof(double);
  double* d = reinterpret_cast<double*>(&s);
#pragma unroll
  for (int k = 0; k < n; k++) d[k] = state[k * nq_total + gq];
}
template <typename State>
SFX_HDI void store_state(const State& s, double* state, int64_t gq, int64_t nq_total) {
  constexpr int n = sizeof(State) / sizeof(double);
  const double* d = reinterpret_cast<const double*>(&s);
#pragma unroll
  for (int k = 0; k < n; k++) state[k * nq_total + gq] = d[k];
}

/// Residual / JVP over a batch of elements.
///   QFMaker: callable (const double* params_of_element) -> q-function for that element
template <int P, int C, int MODE, typename Real, typename State, typename QFMaker>
__global__ void __launch_bounds__(128) domain_kernel(DomainArgs<Real> a, QFMaker make_qf) {
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q * Q;
  constexpr int EPW = 32 / NQ;  // elements per warp
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

  __shared__ Real sB[Q][Q], sD[Q][Q];
  if (threadIdx.x < Q * Q) {
    int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = Real(basis_table<P>().B[i][j]);
    sD[i][j] = Real(basis_table<P>().D[i][j]);
  }
  __syncthreads();

  const int64_t nq_total = a.num_elements * NQ;
  const int64_t gq = e * NQ + qi;
  int32_t node = valid ? a.conn[e * NQ + qi] : 0;

  // interpolate u (and du) at this lane's point
  value_t<C, Real> uv{}, dv{};
  grad_t<C, Real> ug{}, dg{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    Real g[3];
    interpolate_colloc<Q, Real>(U, base, ix, iy, iz, sB, sD, comp<C>(uv, c), g[0], g[1], g[2]);
    for (int j = 0; j < 3; j++) comp<C>(ug, c)[j] = g[j];
    if constexpr (MODE == JVP) {
      Real dU = valid ? a.du[c * a.num_nodes + node] : Real(0);
      interpolate_colloc<Q, Real>(dU, base, ix, iy, iz, sB, sD, comp<C>(dv, c), g[0], g[1], g[2]);
      for (int j = 0; j < 3; j++) comp<C>(dg, c)[j] = g[j];
    }
  }

  // geometric factors
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

  // parent -> physical gradients (finite_element.hpp:246-273)
  using S = std::conditional_t<MODE == JVP, dual<Real, Real>, Real>;
  value_t<C, S> qv{};
  grad_t<C, S> qg{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    if constexpr (MODE == JVP) {
      comp<C>(qv, c) = S{comp<C>(uv, c), comp<C>(dv, c)};
    } else {
      comp<C>(qv, c) = comp<C>(uv, c);
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Real gu = comp<C>(ug, c)[0] * Ji[0][j] + comp<C>(ug, c)[1] * Ji[1][j] + comp<C>(ug, c)[2] * Ji[2][j];
      if constexpr (MODE == JVP) {
        Real gd = comp<C>(dg, c)[0] * Ji[0][j] + comp<C>(dg, c)[1] * Ji[1][j] + comp<C>(dg, c)[2] * Ji[2][j];
        comp<C>(qg, c)[j] = S{gu, gd};
      } else {
        comp<C>(qg, c)[j] = gu;
      }
    }
  }

  // q-function
  const auto qf = make_qf(a.params + (valid ? e : 0) * QFMaker::nparams);
  auto position = tuple{X, Jm};
  auto arg = tuple{qv, qg};
  auto call = [&]() {
    if constexpr (std::is_same<State, Nothing>::value) {
      return qf(a.t, position, arg);
    } else {
      State st{};
      if (valid) load_state(st, a.state, gq, nq_total);
      auto r = qf(a.t, position, st, arg);
      if constexpr (MODE == RESIDUAL_UPDATE) {
        if (valid) store_state(st, a.state, gq, nq_total);
      }
      return r;
    }
  };
  auto out = call();
  using SrcT = std::decay_t<decltype(get<0>(out))>;
  using FluxT = std::decay_t<decltype(get<1>(out))>;
  constexpr bool HS = has_part<MODE, SrcT>();
  constexpr bool HF = has_part<MODE, FluxT>();

  // physical -> parent (finite_element.hpp:287-322), weight folded into dvol,
  // then integrate each component
  Real* out_e = a.out_e + e * (C * NQ);
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real s = 0, f[3] = {0, 0, 0};
    if constexpr (HS) s = dvol * part<MODE, Real>(source_comp<C>(get<0>(out), c));
    if constexpr (HF) {
      auto frow = flux_row<C>(get<1>(out), c);
      Real fp[3];
#pragma unroll
      for (int m = 0; m < 3; m++) fp[m] = part<MODE, Real>(frow[m]);
#pragma unroll
      for (int k = 0; k < 3; k++) f[k] = dvol * (fp[0] * Ji[k][0] + fp[1] * Ji[k][1] + fp[2] * Ji[k][2]);
    }
    Real r = integrate_colloc<Q, HS, HF, Real>(s, f[0], f[1], f[2], base, ix, iy, iz, sB, sD);
    if (valid) out_e[c * NQ + qi] = r;
  }
}

/// Derivative of the shape-aware residual with respect to the shape
/// displacement, applied to a direction dp (serac's ShapeAwareFunctional
/// differentiated with respect to argument 0, shape_aware_functional.hpp:537-541):
/// the geometry is recomputed at each point from the element's vertices Xe
/// ([e][3][8]) and the shape field p (nullptr = 0) with dual numbers carrying
/// dp, x' = X + p + eps dp and dx'/dxi = J + dp/dxi + eps d(dp)/dxi, so that
/// (dx'/dxi)^-1, det(dx'/dxi), the trial gradient du/dx' and the q-function
/// output all carry their directional derivatives; the derivative part of the
/// integrand is integrated into out_e [e][c][node].  a.u holds u, a.geom is
/// not used; quadrature state is read, never written.
template <int P, int C, typename State, typename QFMaker>
__global__ void __launch_bounds__(128) shape_jvp_kernel(DomainArgs<double> a, QFMaker make_qf,
                                                        const double* __restrict__ Xe,
                                                        const double* __restrict__ shape,
                                                        const double* __restrict__ dshape) {
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

  // trial field, shape field and shape direction at this lane's point
  value_t<C, Real> uv{};
  grad_t<C, Real> ug{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    Real g[3];
    interpolate_lane<Q, Real>(U, base, ix, iy, iz, sB, sG, comp<C>(uv, c), g[0], g[1], g[2]);
    for (int j = 0; j < 3; j++) comp<C>(ug, c)[j] = g[j];
  }
  tensor<S, 3> xs{};
  tensor<S, 3, 3> Js{};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    Real pv = 0, pg[3] = {0, 0, 0}, dv = 0, dg[3] = {0, 0, 0};
    Real Pn = (valid && shape) ? shape[i * a.num_nodes + node] : Real(0);
    Real dPn = valid ? dshape[i * a.num_nodes + node] : Real(0);
    interpolate_lane<Q, Real>(Pn, base, ix, iy, iz, sB, sG, pv, pg[0], pg[1], pg[2]);
    interpolate_lane<Q, Real>(dPn, base, ix, iy, iz, sB, sG, dv, dg[0], dg[1], dg[2]);
    xs[i] = S{pv, dv};
#pragma unroll
    for (int j = 0; j < 3; j++) Js[i][j] = S{pg[j], dg[j]};
  }
  // reference (trilinear) geometry at the point
  const Real sp[3] = {gl_point(Q, ix), gl_point(Q, iy), gl_point(Q, iz)};
  const Real w = gl_weight(Q, ix) * gl_weight(Q, iy) * gl_weight(Q, iz);
  const Real* Xv = Xe + (valid ? e : 0) * 24;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const int b0 = v & 1, b1 = (v >> 1) & 1, b2 = (v >> 2) & 1;
    const Real N0 = b0 ? sp[0] : 1.0 - sp[0], N1 = b1 ? sp[1] : 1.0 - sp[1], N2 = b2 ? sp[2] : 1.0 - sp[2];
    const Real d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0, d2 = b2 ? 1.0 : -1.0;
    const Real phi = N0 * N1 * N2;
    const Real g[3] = {d0 * N1 * N2, N0 * d1 * N2, N0 * N1 * d2};
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const Real xv = Xv[i * 8 + v];
      xs[i].value += xv * phi;
#pragma unroll
      for (int j = 0; j < 3; j++) Js[i][j].value += xv * g[j];
    }
  }
  if (!valid) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) Js[i][j] = S{Real(i == j), Real(0)};
  }
  const auto Jinv = inv(Js);
  const S dvol = det(Js) * w;

  // trial gradient in the shape-displaced configuration: du/dxi (dx'/dxi)^-1
  value_t<C, S> qv{};
  grad_t<C, S> qg{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    comp<C>(qv, c) = S{comp<C>(uv, c), Real(0)};
#pragma unroll
    for (int j = 0; j < 3; j++)
      comp<C>(qg, c)[j] = comp<C>(ug, c)[0] * Jinv[0][j] + comp<C>(ug, c)[1] * Jinv[1][j] +
                          comp<C>(ug, c)[2] * Jinv[2][j];
  }
  const auto qf = make_qf(a.params + (valid ? e : 0) * QFMaker::nparams);
  auto position = tuple{xs, Js};
  auto arg = tuple{qv, qg};
  auto call = [&]() {
    if constexpr (std::is_same<State, Nothing>::value) {
      return qf(a.t, position, arg);
    } else {
      State st{};
      if (valid) load_state(st, a.state, gq, nq_total);
      return qf(a.t, position, st, arg);
    }
  };
  auto out = call();
  using SrcT = std::decay_t<decltype(get<0>(out))>;
  using FluxT = std::decay_t<decltype(get<1>(out))>;
  constexpr bool HSrc = !is_zero<typename base_scalar<SrcT>::type>::value;
  constexpr bool HFlx = !is_zero<typename base_scalar<FluxT>::type>::value;
  Real* out_e = a.out_e + e * (C * NQ);
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real src = 0, f[3] = {0, 0, 0};
    if constexpr (HSrc) src = part<JVP, Real>(dvol * source_comp<C>(get<0>(out), c));
    if constexpr (HFlx) {
      auto frow = flux_row<C>(get<1>(out), c);
#pragma unroll
      for (int k = 0; k < 3; k++) f[k] = part<JVP, Real>(dvol * (frow[0] * Jinv[k][0] + frow[1] * Jinv[k][1] + frow[2] * Jinv[k][2]));
    }
    Real r = integrate_lane<Q, HSrc, HFlx, Real>(src, f[0], f[1], f[2], base, ix, iy, iz, sB, sG);
    if (valid) out_e[c * NQ + qi] = r;
  }
}

/// The node-owner scatter of a structured mesh (elements e = ex + nx (ey +
/// ny ez), nodes x + Nx (y + Ny z), Nx = P nx + 1): the elements containing
/// a node and its local index follow from its grid position, so no node ->
/// element table is read, and blocks of 32 x 8 nodes of one node plane read
/// the element vectors of a compact patch.  Sums in increasing element order,
/// as scatter_kernel, so the result is bitwise that of scatter_kernel.
/// Node planes [z0, z1) (blockIdx.z + z0).
template <int P, int C, typename Real>
__global__ void __launch_bounds__(256) grid_scatter_kernel(const Real* __restrict__ E, Real* __restrict__ out,
                                                           int nx, int ny, int nz, bool accumulate, int z0) {
  constexpr int n = P + 1;
  constexpr int NPE = n * n * n;
  const int Nx = P * nx + 1, Ny = P * ny + 1;
  const int x = int(blockIdx.x) * 32 + int(threadIdx.x & 31), y = int(blockIdx.y) * 8 + int(threadIdx.x >> 5);
  const int z = z0 + int(blockIdx.z);
  if (x >= Nx || y >= Ny) return;
  const int64_t num_nodes = int64_t(Nx) * Ny * (int64_t(P) * nz + 1);
  const int64_t node = x + int64_t(Nx) * (y + int64_t(Ny) * z);
  // per direction: the (element, local index) pairs containing the node,
  // lower element first (slot 0 below slot 1; a node inside an element has
  // slot 0 only)
  const int I[3] = {x, y, z}, dims[3] = {nx, ny, nz};
  int el[3][2], lo[3][2];
  bool ok[3][2];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int e = I[d] / P, r = I[d] - e * P;
    el[d][0] = r == 0 ? e - 1 : e;
    lo[d][0] = r == 0 ? P : r;
    ok[d][0] = r != 0 || e > 0;
    el[d][1] = e;
    lo[d][1] = 0;
    ok[d][1] = r == 0 && e < dims[d];
  }
  Real acc[C];
#pragma unroll
  for (int c = 0; c < C; c++) acc[c] = accumulate ? out[c * num_nodes + node] : Real(0);
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int k = 0; k < 2; k++) {
        if (!(ok[2][a] && ok[1][b] && ok[0][k])) continue;
        const int64_t e = el[0][k] + int64_t(nx) * (el[1][b] + int64_t(ny) * el[2][a]);
        const int loc = lo[0][k] + n * (lo[1][b] + n * lo[2][a]);
#pragma unroll
        for (int c = 0; c < C; c++) acc[c] += E[(e * C + c) * NPE + loc];
      }
#pragma unroll
  for (int c = 0; c < C; c++) out[c * num_nodes + node] = acc[c];
}

/// L[c * N + node] (+)= sum over the node's (element, local node) pairs, in
/// element order, of E[(e * C + c) * NPE + local], for the nodes
/// [node_begin, node_end).  One thread per node.
template <int C, int NPE, typename Real>
__global__ void __launch_bounds__(256) scatter_kernel(const Real* __restrict__ E, const int32_t* __restrict__ node_ptr,
                                                      const int32_t* __restrict__ node_ent, Real* __restrict__ out,
                                                      int64_t num_nodes, bool accumulate, int64_t node_begin,
                                                      int64_t node_end) {
  const int64_t n = node_begin + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= node_end) return;
  int32_t b = node_ptr[n], end = node_ptr[n + 1];
  Real acc[C];
#pragma unroll
  for (int c = 0; c < C; c++) acc[c] = accumulate ? out[c * num_nodes + n] : Real(0);
  for (int32_t k = b; k < end; k++) {
    int32_t ent = node_ent[k];
    int64_t el = ent / NPE;
    int32_t loc = ent - int32_t(el) * NPE;
#pragma unroll
    for (int c = 0; c < C; c++) acc[c] += E[(el * C + c) * NPE + loc];
  }
#pragma unroll
  for (int c = 0; c < C; c++) out[c * num_nodes + n] = acc[c];
}

}  // namespace kernels
}  // namespace sfx

namespace sfx {
namespace kernels {

/// Geometric factors of trilinear hexahedra at the Q^3 Gauss points
/// (geometric_factors.cpp:17-60 computes X and J; the inverse, det(J) and the
/// quadrature weight are folded here once instead of at every evaluation).
/// Xe: [e][3][8] lexicographic vertex coordinates.  One thread per point.
template <int Q>
__global__ void __launch_bounds__(256) geometry_kernel(const double* __restrict__ Xe, double* __restrict__ g64,
                                                       float* __restrict__ g32, int64_t ne) {
  constexpr int NQ = Q * Q * Q;
  const int64_t nqt = ne * NQ;
  int64_t gq = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gq >= nqt) return;
  int64_t e = gq / NQ;
  int q = int(gq - e * NQ);
  int qx = q % Q, qy = (q / Q) % Q, qz = q / (Q * Q);
  double s[3] = {gl_point(Q, qx), gl_point(Q, qy), gl_point(Q, qz)};
  double w = gl_weight(Q, qx) * gl_weight(Q, qy) * gl_weight(Q, qz);
  const double* X = Xe + e * 24;
  tensor<double, 3> x{};
  tensor<double, 3, 3> J{};
  for (int v = 0; v < 8; v++) {
    int b0 = v & 1, b1 = (v >> 1) & 1, b2 = (v >> 2) & 1;
    double N0 = b0 ? s[0] : 1.0 - s[0], N1 = b1 ? s[1] : 1.0 - s[1], N2 = b2 ? s[2] : 1.0 - s[2];
    double d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0, d2 = b2 ? 1.0 : -1.0;
    double phi = N0 * N1 * N2;
    double g[3] = {d0 * N1 * N2, N0 * d1 * N2, N0 * N1 * d2};
    for (int i = 0; i < 3; i++) {
      double xv = X[i * 8 + v];
      x[i] += xv * phi;
      for (int j = 0; j < 3; j++) J[i][j] += xv * g[j];
    }
  }
  auto Ji = inv(J);
  double dv = det(J) * w;
  double vals[GEOM_STRIDE];
  for (int k = 0; k < 9; k++) vals[k] = Ji[k / 3][k % 3];
  vals[9] = dv;
  for (int k = 0; k < 3; k++) vals[10 + k] = x[k];
  for (int k = 0; k < 9; k++) vals[13 + k] = J[k / 3][k % 3];
  for (int k = 0; k < GEOM_STRIDE; k++) {
    g64[k * nqt + gq] = vals[k];
    g32[k * nqt + gq] = float(vals[k]);
  }
}

/// Geometric factors of the shape-displaced configuration x' = X + p
/// (serac's ShapeAwareFunctional, shape_aware_functional.hpp:45-120): p is a
/// 3-component H1 field of order P on the form's node grid (byNODES,
/// shape[i * num_nodes + node]); dx'/dxi = dX/dxi + dp/dxi.  Evaluating the
/// plain element kernels with these factors gives serac's corrections
/// du/dx' = du/dX (I + dp/dX)^-1, flux (I + dp/dX)^-T det(I + dp/dX) and
/// source det(I + dp/dX).  One thread per quadrature point; same layout as
/// geometry_kernel.
template <int P>
__global__ void __launch_bounds__(256) geometry_shape_kernel(const double* __restrict__ Xe,
                                                             const int32_t* __restrict__ conn,
                                                             const double* __restrict__ shape, int64_t num_nodes,
                                                             double* __restrict__ g64, float* __restrict__ g32,
                                                             int64_t ne) {
  constexpr int Q = P + 1, NQ = Q * Q * Q, N1 = P + 1, NPE = N1 * N1 * N1;
  const int64_t nqt = ne * NQ;
  int64_t gq = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gq >= nqt) return;
  int64_t e = gq / NQ;
  int q = int(gq - e * NQ);
  int qx = q % Q, qy = (q / Q) % Q, qz = q / (Q * Q);
  double s[3] = {gl_point(Q, qx), gl_point(Q, qy), gl_point(Q, qz)};
  double w = gl_weight(Q, qx) * gl_weight(Q, qy) * gl_weight(Q, qz);
  const double* X = Xe + e * 24;
  tensor<double, 3> x{};
  tensor<double, 3, 3> J{};
  for (int v = 0; v < 8; v++) {
    int b0 = v & 1, b1 = (v >> 1) & 1, b2 = (v >> 2) & 1;
    double N0 = b0 ? s[0] : 1.0 - s[0], N1v = b1 ? s[1] : 1.0 - s[1], N2 = b2 ? s[2] : 1.0 - s[2];
    double d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0, d2 = b2 ? 1.0 : -1.0;
    double phi = N0 * N1v * N2;
    double g[3] = {d0 * N1v * N2, N0 * d1 * N2, N0 * N1v * d2};
    for (int i = 0; i < 3; i++) {
      double xv = X[i * 8 + v];
      x[i] += xv * phi;
      for (int j = 0; j < 3; j++) J[i][j] += xv * g[j];
    }
  }
  const auto& T = basis_table<P>();
  const int32_t* ce = conn + e * NPE;
  for (int a = 0; a < NPE; a++) {
    const int ax = a % N1, ay = (a / N1) % N1, az = a / (N1 * N1);
    const double bx = T.B[qx][ax], by = T.B[qy][ay], bz = T.B[qz][az];
    const double phi = bx * by * bz;
    const double g[3] = {T.G[qx][ax] * by * bz, bx * T.G[qy][ay] * bz, bx * by * T.G[qz][az]};
    const int64_t node = ce[a];
    for (int i = 0; i < 3; i++) {
      const double pv = shape[i * num_nodes + node];
      x[i] += pv * phi;
      for (int j = 0; j < 3; j++) J[i][j] += pv * g[j];
    }
  }
  auto Ji = inv(J);
  double dv = det(J) * w;
  double vals[GEOM_STRIDE];
  for (int k = 0; k < 9; k++) vals[k] = Ji[k / 3][k % 3];
  vals[9] = dv;
  for (int k = 0; k < 3; k++) vals[10 + k] = x[k];
  for (int k = 0; k < 9; k++) vals[13 + k] = J[k / 3][k % 3];
  for (int k = 0; k < GEOM_STRIDE; k++) {
    g64[k * nqt + gq] = vals[k];
    g32[k * nqt + gq] = float(vals[k]);
  }
}

}  // namespace kernels
}  // namespace sfx

namespace sfx {
namespace kernels {

/// Element stiffness matrices dR_e/du_e at the linearisation point, stored
/// K[e][trial vdof][test vdof] like serac's element_gradient_kernel
/// (domain_integral_kernels.hpp:327-361; vdof = component * NPE + node).
/// Lane q first linearises the q-function at its point one trial component
/// at a time (4 directional dual evaluations seeded on the parent-space value
/// and gradient, giving the 4C x 4 block of the derivative), then for every
/// trial node j applies that block to (phi_j, grad_xi phi_j) at its point and
/// integrates with the transposed sum-factorised passes, so that lane i ends
/// with K[(cj, j)][(ci, i)].  diag_only: only the diagonal entries, written to
/// an E-vector [e][c][node].
template <int P, int C, typename State, typename QFMaker, bool diag_only>
__global__ void __launch_bounds__(128) element_matrix_kernel(DomainArgs<double> a, QFMaker make_qf, int64_t e_begin,
                                                             int64_t e_end) {
  using Real = double;
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q * Q;
  constexpr int EPW = 32 / NQ;
  constexpr int NDOF = C * NQ;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / NQ;
  const int qi_raw = lane - sub * NQ;
  const bool slot = sub < EPW;
  const int qi = slot ? qi_raw : NQ - 1;
  const int base = slot ? sub * NQ : 0;
  const int64_t e = e_begin + warp * EPW + (slot ? sub : 0);
  const bool valid = slot && e < e_end;
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
  const int64_t el = e - e_begin;  // slot in the output chunk
  int32_t node = valid ? a.conn[e * NQ + qi] : 0;

  value_t<C, Real> uv{};
  grad_t<C, Real> ug{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    Real g[3];
    interpolate_lane<Q, Real>(U, base, ix, iy, iz, sB, sG, comp<C>(uv, c), g[0], g[1], g[2]);
    for (int j = 0; j < 3; j++) comp<C>(ug, c)[j] = g[j];
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
  // physical gradient of u
  Real gx[C][3];
#pragma unroll
  for (int c = 0; c < C; c++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      gx[c][j] = comp<C>(ug, c)[0] * Ji[0][j] + comp<C>(ug, c)[1] * Ji[1][j] + comp<C>(ug, c)[2] * Ji[2][j];

  const auto qf = make_qf(a.params + (valid ? e : 0) * QFMaker::nparams);
  auto position = tuple{X, Jm};
  State st0{};
  if constexpr (!std::is_same<State, Nothing>::value) {
    if (valid) load_state(st0, a.state, gq, nq_total);
  }
  using S = dual<Real, Real>;

#pragma unroll 1
  for (int cj = 0; cj < C; cj++) {
    // D[out][b]: derivative of parent-space output `out` (source ci, flux ci*3+k)
    // w.r.t. the parent-space input b of component cj (0: value, 1..3: d/dxi_k)
    Real Ds[C][4];
    Real Df[C][3][4];
#pragma unroll
    for (int b = 0; b < 4; b++) {
      value_t<C, S> qv{};
      grad_t<C, S> qg{};
#pragma unroll
      for (int c = 0; c < C; c++) {
        comp<C>(qv, c) = S{comp<C>(uv, c), Real(c == cj && b == 0)};
#pragma unroll
        for (int j = 0; j < 3; j++) comp<C>(qg, c)[j] = S{gx[c][j], (c == cj && b > 0) ? Ji[b - 1][j] : Real(0)};
      }
      auto arg = tuple{qv, qg};
      auto call = [&]() {
        if constexpr (std::is_same<State, Nothing>::value) {
          return qf(a.t, position, arg);
        } else {
          State st = st0;
          return qf(a.t, position, st, arg);
        }
      };
      auto out = call();
      using SrcT = std::decay_t<decltype(get<0>(out))>;
      using FluxT = std::decay_t<decltype(get<1>(out))>;
#pragma unroll
      for (int ci = 0; ci < C; ci++) {
        if constexpr (has_part<JVP, SrcT>()) Ds[ci][b] = dvol * part<JVP, Real>(source_comp<C>(get<0>(out), ci));
        else Ds[ci][b] = 0;
        if constexpr (has_part<JVP, FluxT>()) {
          auto frow = flux_row<C>(get<1>(out), ci);
          Real fp[3];
#pragma unroll
          for (int m = 0; m < 3; m++) fp[m] = part<JVP, Real>(frow[m]);
#pragma unroll
          for (int k = 0; k < 3; k++) Df[ci][k][b] = dvol * (fp[0] * Ji[k][0] + fp[1] * Ji[k][1] + fp[2] * Ji[k][2]);
        } else {
#pragma unroll
          for (int k = 0; k < 3; k++) Df[ci][k][b] = 0;
        }
      }
    }
    if constexpr (diag_only) {
      // K[(cj,i)][(cj,i)] = sum_q Psi_i(q)^T D Psi_i(q): each lane needs every
      // point's contribution for its own node: integrate with trial node = test node
#pragma unroll 1
      for (int j = 0; j < NQ; j++) {
        const int jx = j % Q, jy = (j / Q) % Q, jz = j / (Q * Q);
        Real psi[4] = {sB[ix][jx] * sB[iy][jy] * sB[iz][jz], sG[ix][jx] * sB[iy][jy] * sB[iz][jz],
                       sB[ix][jx] * sG[iy][jy] * sB[iz][jz], sB[ix][jx] * sB[iy][jy] * sG[iz][jz]};
        Real s = Ds[cj][0] * psi[0] + Ds[cj][1] * psi[1] + Ds[cj][2] * psi[2] + Ds[cj][3] * psi[3];
        Real f[3];
#pragma unroll
        for (int k = 0; k < 3; k++)
          f[k] = Df[cj][k][0] * psi[0] + Df[cj][k][1] * psi[1] + Df[cj][k][2] * psi[2] + Df[cj][k][3] * psi[3];
        Real r = integrate_lane<Q, true, true, Real>(s, f[0], f[1], f[2], base, ix, iy, iz, sB, sG);
        if (valid && qi == j) a.out_e[(e * C + cj) * NQ + qi] = r;  // diagonal E-vector covers all elements
      }
    } else {
#pragma unroll 1
      for (int j = 0; j < NQ; j++) {
        const int jx = j % Q, jy = (j / Q) % Q, jz = j / (Q * Q);
        Real psi[4] = {sB[ix][jx] * sB[iy][jy] * sB[iz][jz], sG[ix][jx] * sB[iy][jy] * sB[iz][jz],
                       sB[ix][jx] * sG[iy][jy] * sB[iz][jz], sB[ix][jx] * sB[iy][jy] * sG[iz][jz]};
        Real* col = a.out_e + (el * NDOF + (cj * NQ + j)) * int64_t(NDOF);
#pragma unroll
        for (int ci = 0; ci < C; ci++) {
          Real s = Ds[ci][0] * psi[0] + Ds[ci][1] * psi[1] + Ds[ci][2] * psi[2] + Ds[ci][3] * psi[3];
          Real f[3];
#pragma unroll
          for (int k = 0; k < 3; k++)
            f[k] = Df[ci][k][0] * psi[0] + Df[ci][k][1] * psi[1] + Df[ci][k][2] * psi[2] + Df[ci][k][3] * psi[3];
          Real r = integrate_lane<Q, true, true, Real>(s, f[0], f[1], f[2], base, ix, iy, iz, sB, sG);
          if (valid) col[ci * NQ + qi] = r;
        }
      }
    }
  }
}

/// CSR graph of a structured-mesh H1 form: row (comp, node) holds, for every
/// component, the box of nodes covered by the elements that contain the node
/// (the union of their nodes is the product of three 1-D index ranges).
struct GridShape {
  int p;
  int64_t N[3];   // nodes per direction
  int64_t ne[3];  // elements per direction
  struct Row {
    int64_t lo[3], w[3], len;
  };
  SFX_HDI int64_t num_nodes() const { return N[0] * N[1] * N[2]; }
  SFX_HDI void range(int d, int64_t I, int64_t& lo, int64_t& hi) const {
    if (I % p == 0) {
      const int64_t e = I / p;
      lo = (e > 0) ? I - p : I;
      hi = (e < ne[d]) ? I + p : I;
    } else {
      const int64_t e = I / p;
      lo = e * p;
      hi = e * p + p;
    }
  }
  SFX_HDI Row row(int64_t node) const {
    const int64_t I[3] = {node % N[0], (node / N[0]) % N[1], node / (N[0] * N[1])};
    Row r{};
    for (int d = 0; d < 3; d++) {
      int64_t hi = 0;
      range(d, I[d], r.lo[d], hi);
      r.w[d] = hi - r.lo[d] + 1;
    }
    r.len = r.w[0] * r.w[1] * r.w[2];
    return r;
  }
  /// k-th scalar column of the row (ascending node ids)
  SFX_HDI int64_t column(const Row& r, int64_t k) const {
    const int64_t x = r.lo[0] + k % r.w[0], y = r.lo[1] + (k / r.w[0]) % r.w[1], z = r.lo[2] + k / (r.w[0] * r.w[1]);
    return x + N[0] * (y + N[1] * z);
  }
  /// position of node nb among the row's scalar columns
  SFX_HDI int64_t pos(const Row& r, int64_t nb) const {
    const int64_t x = nb % N[0], y = (nb / N[0]) % N[1], z = nb / (N[0] * N[1]);
    return ((z - r.lo[2]) * r.w[1] + (y - r.lo[1])) * r.w[0] + (x - r.lo[0]);
  }
};

/// CSR graph of a form built from an imported element table: the sorted
/// scalar adjacency (the union of the nodes of a node's elements) per node,
/// columns located by binary search.
struct TableGraph {
  const int64_t* sptr;  // [num_nodes + 1]
  const int32_t* scol;  // ascending within each row
  int64_t nn;
  struct Row {
    int64_t begin, len;
  };
  SFX_HDI int64_t num_nodes() const { return nn; }
  SFX_HDI Row row(int64_t node) const { return {sptr[node], sptr[node + 1] - sptr[node]}; }
  SFX_HDI int64_t column(const Row& r, int64_t k) const { return scol[r.begin + k]; }
  SFX_HDI int64_t pos(const Row& r, int64_t nb) const {
    int64_t lo = 0, hi = r.len - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (scol[r.begin + mid] < nb) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  }
};

template <int C, typename Graph>
__global__ void csr_row_length_kernel(Graph g, int64_t* row_len) {
  const int64_t nn = g.num_nodes();
  int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= nn * C) return;
  row_len[r + 1] = int64_t(C) * g.row(r % nn).len;
  if (r == 0) row_len[0] = 0;
}

template <int C, typename Graph>
__global__ void csr_fill_kernel(Graph g, const int64_t* __restrict__ row_ptr, int32_t* __restrict__ col) {
  const int64_t nn = g.num_nodes();
  int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= nn * C) return;
  const auto row = g.row(r % nn);
  int64_t k = row_ptr[r];
  for (int c = 0; c < C; c++)
    for (int64_t j = 0; j < row.len; j++) col[k++] = int32_t(c * nn + g.column(row, j));
}

/// values[row] = sum over the row node's elements (element order) of the
/// element-matrix entries; one thread per row, so the order of the additions
/// is fixed.  Ke: [e][trial vdof][test vdof].
template <int P, int C, typename Graph>
__global__ void csr_assemble_kernel(Graph g, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ conn,
                                    const int32_t* __restrict__ node_ptr, const int32_t* __restrict__ node_ent,
                                    const double* __restrict__ Ke, int64_t e_begin, int64_t e_end,
                                    double* __restrict__ values, bool accumulate) {
  constexpr int NPE = (P + 1) * (P + 1) * (P + 1);
  constexpr int NDOF = C * NPE;
  const int64_t nn = g.num_nodes();
  int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= nn * C) return;
  const int ci = int(r / nn);
  const int64_t node = r - ci * nn;
  const auto grow = g.row(node);
  const int64_t scalar_len = grow.len;
  double* row = values + row_ptr[r];
  if (!accumulate)
    for (int64_t k = 0; k < C * scalar_len; k++) row[k] = 0.0;
  for (int32_t t = node_ptr[node]; t < node_ptr[node + 1]; t++) {
    const int32_t ent = node_ent[t];
    const int64_t e = ent / NPE;
    if (e < e_begin || e >= e_end) continue;
    const int a = ent - int(e) * NPE;
    const double* Kcol = Ke + (e - e_begin) * NDOF * NDOF + (ci * NPE + a);  // stride NDOF over trial vdofs
    for (int b = 0; b < NPE; b++) {
      const int64_t pos = g.pos(grow, conn[e * NPE + b]);
#pragma unroll
      for (int cj = 0; cj < C; cj++) row[cj * scalar_len + pos] += Kcol[int64_t(cj * NPE + b) * NDOF];
    }
  }
}

}  // namespace kernels
}  // namespace sfx

namespace sfx {
namespace kernels {

template <typename State, typename QF, typename Pos, typename Arg>
SFX_HDI auto invoke_qf(const QF& qf, double t, const Pos& pos, State& st, const Arg& arg) {
  if constexpr (std::is_same<State, Nothing>::value) {
    (void)st;
    return qf(t, pos, arg);
  } else {
    return qf(t, pos, st, arg);
  }
}

/// Whether the q-function's source output depends on the trial field (the
/// stored derivative then has source rows).
template <int C, typename State, typename QF>
constexpr bool tangent_has_source() {
  using S = dual<double, double>;
  using Out = decltype(invoke_qf<State>(std::declval<const QF&>(), 0.0,
                                        std::declval<tuple<tensor<double, 3>, tensor<double, 3, 3>>>(),
                                        std::declval<State&>(), std::declval<tuple<value_t<C, S>, grad_t<C, S>>>()));
  using SrcT = std::decay_t<decltype(get<0>(std::declval<Out>()))>;
  return has_part<JVP, SrcT>();
}

/// Shape of the stored q-function derivative per quadrature point:
/// rows = parent-space outputs (source components if the source depends on the
/// trial field, then the C x 3 flux), cols = parent-space inputs (values if the
/// q-function reads them, then the C x 3 gradient).  SYM: the block is
/// symmetric (a hyperelastic or associative-plastic tangent, whose flux is
/// the gradient of a potential in the trial gradient; det(J) w and the
/// parent-space map J^-1 (.) J^-T keep that symmetry), so only its upper
/// triangle is stored, row-major (packed): 45 entries instead of 81 for the
/// vector 9 x 9 block, 6 instead of 9 for the scalar 3 x 3 one.
template <int C, bool HS, bool VI, bool SYM = false>
struct TangentShape {
  static constexpr int rows = (HS ? C : 0) + 3 * C;
  static constexpr int cols = (VI ? C : 0) + 3 * C;
  static constexpr bool packed = SYM && rows == cols;
  static constexpr int size = packed ? rows * (rows + 1) / 2 : rows * cols;
  /// position of entry (r, k) in the per-point block (packed: r <= k)
  static SFX_HDI constexpr int index(int r, int k) {
    return packed ? r * cols - r * (r - 1) / 2 + (k - r) : r * cols + k;
  }
  /// entries of one element's block (size x NQ) rounded up to a multiple of
  /// 4, so that every block starts on a 16-byte (FP32) / 32-byte (FP64)
  /// boundary and can be moved by a bulk copy
  template <int NQ>
  static constexpr int64_t stride = (int64_t(size) * NQ + 3) / 4 * 4;
  /// row and column of entry m of the per-point block (the inverse of index)
  static SFX_HDI constexpr int row_of(int m) {
    if (!packed) return m / cols;
    int r = 0;
    while (m >= cols - r) {
      m -= cols - r;
      r++;
    }
    return r;
  }
  static SFX_HDI constexpr int col_of(int m) {
    if (!packed) return m % cols;
    int r = 0;
    while (m >= cols - r) {
      m -= cols - r;
      r++;
    }
    return r + m;
  }
  /// entry pairs per point of the FP16 copy
  static constexpr int pairs = (size + 1) / 2;
  /// the FP16 copy stores entries (2j, 2j + 1) of a point next to each other
  /// (one half2 per lane and pair): position of entry m of point q in an
  /// element's block
  template <int NQ>
  static SFX_HDI constexpr int64_t pos16(int m, int q) {
    return (int64_t(m / 2) * NQ + q) * 2 + (m & 1);
  }
  /// the same for the FP16 copy (pairs x NQ half2, multiples of 8 halves = 16 bytes)
  template <int NQ>
  static constexpr int64_t stride16 = (int64_t(pairs) * 2 * NQ + 7) / 8 * 8;
  /// entries per element block in storage type TS
  template <int NQ, typename TS>
  static constexpr int64_t stride_of = sizeof(TS) == 2 ? stride16<NQ> : stride<NQ>;
};

/// accumulate entry M (value d) of a point's block into out = D in
/// (TRANSPOSE: D^T in); a packed symmetric entry counts for (r, k) and (k, r)
template <typename Shape, bool TRANSPOSE, int M>
SFX_HDI void tangent_entry(float d, const float* in, float* out) {
  constexpr int r = Shape::row_of(M), k = Shape::col_of(M);
  if constexpr (Shape::packed) {
    out[r] += d * in[k];
    if constexpr (k != r) out[k] += d * in[r];
  } else if constexpr (TRANSPOSE) {
    out[k] += d * in[r];
  } else {
    out[r] += d * in[k];
  }
}

/// out (+)= D in (TRANSPOSE: D^T in) from the FP16 copy, one half2 load per
/// entry pair (entries 2J, 2J + 1 of this point, pair stride NQ)
template <typename Shape, bool TRANSPOSE, int NQ, int... J>
SFX_HDI void apply_pairs16(const __half2* D2, const float* in, float* out, std::integer_sequence<int, J...>) {
  auto pair = [&](auto j) {
    constexpr int jj = decltype(j)::value;
    const float2 d = __half22float2(D2[jj * NQ]);
    tangent_entry<Shape, TRANSPOSE, 2 * jj>(d.x, in, out);
    if constexpr (2 * jj + 1 < Shape::size) tangent_entry<Shape, TRANSPOSE, 2 * jj + 1>(d.y, in, out);
  };
  (pair(std::integral_constant<int, J>{}), ...);
}

/// out = D in (TRANSPOSE: D^T in) for one point's block, read with stride NQ
/// from Dq (this lane's point).  A packed symmetric block is read once per
/// stored entry and used for both (r, k) and (k, r): 45 loads and 81 FMA for
/// the vector 9 x 9 block; D^T = D there.
template <typename Shape, int NQ, bool TRANSPOSE, typename Real, typename TS>
SFX_HDI void apply_block(const TS* Dq, const Real* in, Real* out, bool valid) {
  if constexpr (Shape::packed) {
#pragma unroll
    for (int r = 0; r < Shape::rows; r++) out[r] = Real(0);
#pragma unroll
    for (int r = 0; r < Shape::rows; r++) {
#pragma unroll
      for (int k = r; k < Shape::cols; k++) {
        const Real d = valid ? Real(Dq[Shape::index(r, k) * NQ]) : Real(0);
        out[r] += d * in[k];
        if (k != r) out[k] += d * in[r];
      }
    }
  } else if constexpr (TRANSPOSE) {
#pragma unroll
    for (int k = 0; k < Shape::cols; k++) {
      Real acc = 0;
#pragma unroll
      for (int r = 0; r < Shape::rows; r++) acc += (valid ? Real(Dq[Shape::index(r, k) * NQ]) : Real(0)) * in[r];
      out[k] = acc;
    }
  } else {
#pragma unroll
    for (int r = 0; r < Shape::rows; r++) {
      Real acc = 0;
#pragma unroll
      for (int k = 0; k < Shape::cols; k++) acc += (valid ? Real(Dq[Shape::index(r, k) * NQ]) : Real(0)) * in[k];
      out[r] = acc;
    }
  }
}

/// storage -> FP32 for the tangent copies of the FP32 Jacobian action
SFX_HDI float tangent_to_f32(float x) { return x; }
SFX_HDI float tangent_to_f32(__half x) { return __half2float(x); }

/// Linearise the q-function at every quadrature point (the derivative serac
/// stores in evaluation_kernel_impl, domain_integral_kernels.hpp:209-214, after
/// physical_to_parent, with det(J) w folded in) and, optionally, write the
/// element residuals of the same evaluation.  D is stored element-major,
/// D[e * stride + (row * cols + col) * NQ + q] (stride = TangentShape::stride),
/// in FP64 and FP32 (or FP16 with its own stride16), so that one element's
/// tangent is one contiguous block; D32 / D16 may be null.  SYM: the FP32 /
/// FP16 copies (streamed by the HBM-bound inner action) keep only the upper
/// triangle of a symmetric block; the FP64 copy stays full, because its
/// action is bound by the FP64 pipe, not by the bytes it reads, and the full
/// block keeps one independent accumulation chain per output.
template <int P, int C, typename State, typename QFMaker, bool SYM = false>
__global__ void __launch_bounds__(128) linearize_kernel(DomainArgs<double> a, QFMaker make_qf, double* __restrict__ D64,
                                                        float* __restrict__ D32, __half* __restrict__ D16,
                                                        double* __restrict__ res_e) {
  using Real = double;
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q * Q;
  constexpr int EPW = 32 / NQ;
  constexpr bool VI = QFMaker::value_input;
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
  int32_t node = valid ? a.conn[e * NQ + qi] : 0;

  value_t<C, Real> uv{};
  grad_t<C, Real> ug{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    Real g[3];
    interpolate_lane<Q, Real>(U, base, ix, iy, iz, sB, sG, comp<C>(uv, c), g[0], g[1], g[2]);
    for (int j = 0; j < 3; j++) comp<C>(ug, c)[j] = g[j];
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
  Real gx[C][3];
#pragma unroll
  for (int c = 0; c < C; c++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      gx[c][j] = comp<C>(ug, c)[0] * Ji[0][j] + comp<C>(ug, c)[1] * Ji[1][j] + comp<C>(ug, c)[2] * Ji[2][j];

  const auto qf = make_qf(a.params + (valid ? e : 0) * QFMaker::nparams);
  auto position = tuple{X, Jm};
  State st0{};
  if constexpr (!std::is_same<State, Nothing>::value) {
    if (valid) load_state(st0, a.state, gq, nq_total);
  }
  using S = dual<Real, Real>;
  constexpr int NCOLS = (VI ? C : 0) + 3 * C;

  Real res_s[C] = {}, res_f[C][3] = {};
  bool have_res = false;
#pragma unroll 1
  for (int k = 0; k < NCOLS; k++) {
    // seed: value of component k (k < C when VI), else gradient entry (c, b)
    const int kk = VI ? k : k + C;
    const int seed_c = kk < C ? kk : (kk - C) / 3;
    const int seed_b = kk < C ? -1 : (kk - C) % 3;
    value_t<C, S> qv{};
    grad_t<C, S> qg{};
#pragma unroll
    for (int c = 0; c < C; c++) {
      comp<C>(qv, c) = S{comp<C>(uv, c), Real(c == seed_c && seed_b < 0)};
#pragma unroll
      for (int j = 0; j < 3; j++)
        comp<C>(qg, c)[j] = S{gx[c][j], (c == seed_c && seed_b >= 0) ? Ji[seed_b][j] : Real(0)};
    }
    auto arg = tuple{qv, qg};
    auto call = [&]() {
      if constexpr (std::is_same<State, Nothing>::value) {
        return qf(a.t, position, arg);
      } else {
        State st = st0;
        return qf(a.t, position, st, arg);
      }
    };
    auto out = call();
    using SrcT = std::decay_t<decltype(get<0>(out))>;
    using FluxT = std::decay_t<decltype(get<1>(out))>;
    constexpr bool HS = has_part<JVP, SrcT>();
    using Shape = TangentShape<C, HS, VI>;         // FP64 copy: full block
    using ShapeP = TangentShape<C, HS, VI, SYM>;   // FP32 / FP16 copies: packed when symmetric
    int row = 0;
#pragma unroll
    for (int ci = 0; ci < C; ci++) {
      if constexpr (HS) {
        Real v = dvol * part<JVP, Real>(source_comp<C>(get<0>(out), ci));
        if (valid) {
          D64[e * Shape::template stride<NQ> + int64_t(Shape::index(ci, k)) * NQ + qi] = v;
          if (!ShapeP::packed || ci <= k) {
            const int64_t in_block = int64_t(ShapeP::index(ci, k)) * NQ + qi;
            if (D32) D32[e * ShapeP::template stride<NQ> + in_block] = float(v);
            if (D16)
              D16[e * ShapeP::template stride16<NQ> + ShapeP::template pos16<NQ>(ShapeP::index(ci, k), qi)] =
                  __float2half_rn(float(v));
          }
        }
      }
    }
    row = HS ? C : 0;
#pragma unroll
    for (int ci = 0; ci < C; ci++) {
      Real fp[3] = {0, 0, 0}, fv[3] = {0, 0, 0};
      if constexpr (has_part<JVP, FluxT>()) {
        auto frow = flux_row<C>(get<1>(out), ci);
#pragma unroll
        for (int m = 0; m < 3; m++) fp[m] = part<JVP, Real>(frow[m]);
      }
      if constexpr (has_part<RESIDUAL, FluxT>()) {
        auto frow = flux_row<C>(get<1>(out), ci);
#pragma unroll
        for (int m = 0; m < 3; m++) fv[m] = part<RESIDUAL, Real>(frow[m]);
      }
#pragma unroll
      for (int kd = 0; kd < 3; kd++) {
        Real v = dvol * (fp[0] * Ji[kd][0] + fp[1] * Ji[kd][1] + fp[2] * Ji[kd][2]);
        if (valid) {
          const int rr = row + 3 * ci + kd;
          D64[e * Shape::template stride<NQ> + int64_t(Shape::index(rr, k)) * NQ + qi] = v;
          if (!ShapeP::packed || rr <= k) {
            const int64_t in_block = int64_t(ShapeP::index(rr, k)) * NQ + qi;
            if (D32) D32[e * ShapeP::template stride<NQ> + in_block] = float(v);
            if (D16)
              D16[e * ShapeP::template stride16<NQ> + ShapeP::template pos16<NQ>(ShapeP::index(rr, k), qi)] =
                  __float2half_rn(float(v));
          }
        }
        if (!have_res) res_f[ci][kd] = dvol * (fv[0] * Ji[kd][0] + fv[1] * Ji[kd][1] + fv[2] * Ji[kd][2]);
      }
      if constexpr (has_part<RESIDUAL, SrcT>()) {
        if (!have_res) res_s[ci] = dvol * part<RESIDUAL, Real>(source_comp<C>(get<0>(out), ci));
      }
    }
    have_res = true;
  }
  if (res_e != nullptr) {
    // element residuals of the linearisation point (value part of the evaluation)
#pragma unroll
    for (int c = 0; c < C; c++) {
      Real r = integrate_lane<Q, true, true, Real>(res_s[c], res_f[c][0], res_f[c][1], res_f[c][2], base, ix, iy, iz,
                                                   sB, sG);
      if (valid) res_e[(e * C + c) * NQ + qi] = r;
    }
  }
}

/// Jacobian action from the stored derivative (serac's action_of_gradient_kernel,
/// domain_integral_kernels.hpp:277-304): interpolate du, apply D, integrate.
template <int P, int C, bool HS, bool VI, typename Real, bool SYM = false>
__global__ void __launch_bounds__(128) jvp_stored_kernel(const Real* __restrict__ du, const Real* __restrict__ D,
                                                         const int32_t* __restrict__ conn, Real* __restrict__ out_e,
                                                         int64_t num_nodes, int64_t num_elements) {
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q * Q;
  constexpr int EPW = 32 / NQ;
  using Shape = TangentShape<C, HS, VI, SYM>;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / NQ;
  const int qi_raw = lane - sub * NQ;
  const bool slot = sub < EPW;
  const int qi = slot ? qi_raw : NQ - 1;
  const int base = slot ? sub * NQ : 0;
  const int64_t e = warp * EPW + (slot ? sub : 0);
  const bool valid = slot && e < num_elements;
  const int ix = qi % Q, iy = (qi / Q) % Q, iz = qi / (Q * Q);

  __shared__ Real sB[Q][Q], sD[Q][Q];
  if (threadIdx.x < Q * Q) {
    int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = Real(basis_table<P>().B[i][j]);
    sD[i][j] = Real(basis_table<P>().D[i][j]);
  }
  __syncthreads();

  const int64_t nq_total = num_elements * NQ;
  const int64_t gq = e * NQ + qi;
  const int32_t node = valid ? conn[e * NQ + qi] : 0;

  Real din[Shape::cols];
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? du[c * num_nodes + node] : Real(0);
    Real v, g0, g1, g2;
    interpolate_colloc<Q, Real>(U, base, ix, iy, iz, sB, sD, v, g0, g1, g2);
    if constexpr (VI) din[c] = v;
    constexpr int off = VI ? C : 0;
    din[off + 3 * c + 0] = g0;
    din[off + 3 * c + 1] = g1;
    din[off + 3 * c + 2] = g2;
  }
  Real dout[Shape::rows];
  const Real* Dq = D + (valid ? e * Shape::template stride<NQ> + qi : 0);
  apply_block<Shape, NQ, false>(Dq, din, dout, valid);
  constexpr int roff = HS ? C : 0;
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real s = HS ? dout[HS ? c : 0] : Real(0);
    Real r = integrate_colloc<Q, HS, true, Real>(s, dout[roff + 3 * c], dout[roff + 3 * c + 1], dout[roff + 3 * c + 2],
                                               base, ix, iy, iz, sB, sD);
    if (valid) out_e[(e * C + c) * NQ + qi] = r;
  }
}

/// Transposed Jacobian action from the stored derivative, dr = J^T v (what
/// serac's adjoint solves obtain by transposing the assembled matrix,
/// solid_mechanics.hpp:1343-1501).  D holds, per point, the parent-space block
/// d(outputs)/d(inputs) with det(J) w folded in, so J = B^T D B with B the
/// interpolation to (value, parent gradient); J^T = B^T D^T B: v is
/// interpolated onto the output side (values if the source depends on the
/// field, then the gradient), D^T is applied, and the result is integrated
/// on the input side (values if the q-function reads them, then the flux).
template <int P, int C, bool HS, bool VI, typename Real, bool SYM = false>
__global__ void __launch_bounds__(128) jvp_stored_transpose_kernel(const Real* __restrict__ v,
                                                                   const Real* __restrict__ D,
                                                                   const int32_t* __restrict__ conn,
                                                                   Real* __restrict__ out_e, int64_t num_nodes,
                                                                   int64_t num_elements) {
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q * Q;
  constexpr int EPW = 32 / NQ;
  using Shape = TangentShape<C, HS, VI, SYM>;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / NQ;
  const int qi_raw = lane - sub * NQ;
  const bool slot = sub < EPW;
  const int qi = slot ? qi_raw : NQ - 1;
  const int base = slot ? sub * NQ : 0;
  const int64_t e = warp * EPW + (slot ? sub : 0);
  const bool valid = slot && e < num_elements;
  const int ix = qi % Q, iy = (qi / Q) % Q, iz = qi / (Q * Q);

  __shared__ Real sB[Q][Q], sD[Q][Q];
  if (threadIdx.x < Q * Q) {
    int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = Real(basis_table<P>().B[i][j]);
    sD[i][j] = Real(basis_table<P>().D[i][j]);
  }
  __syncthreads();

  const int32_t node = valid ? conn[e * NQ + qi] : 0;
  constexpr int roff = HS ? C : 0;
  Real vin[Shape::rows];
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real V = valid ? v[c * num_nodes + node] : Real(0);
    Real val, g0, g1, g2;
    interpolate_colloc<Q, Real>(V, base, ix, iy, iz, sB, sD, val, g0, g1, g2);
    if constexpr (HS) vin[c] = val;
    vin[roff + 3 * c + 0] = g0;
    vin[roff + 3 * c + 1] = g1;
    vin[roff + 3 * c + 2] = g2;
  }
  Real vout[Shape::cols];
  const Real* Dq = D + (valid ? e * Shape::template stride<NQ> + qi : 0);
  apply_block<Shape, NQ, true>(Dq, vin, vout, valid);
  constexpr int coff = VI ? C : 0;
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real s = VI ? vout[VI ? c : 0] : Real(0);
    Real r = integrate_colloc<Q, VI, true, Real>(s, vout[coff + 3 * c], vout[coff + 3 * c + 1], vout[coff + 3 * c + 2],
                                               base, ix, iy, iz, sB, sD);
    if (valid) out_e[(e * C + c) * NQ + qi] = r;
  }
}

/// FP32 Jacobian action from the stored tangent for Q2 elements, with each
/// element's tangent block (81 x 27 floats for the vector Neo-Hookean case,
/// 8.7 KB, contiguous) staged into shared memory by bulk asynchronous copies
/// (cp.async.bulk) on mbarriers: each warp owns a ring of STAGES buffers and
/// keeps STAGES - 1 copies in flight while it computes, so the kernel streams
/// the tangent at HBM rate instead of waiting on 81 dependent loads per lane.
/// Elements are dealt to warps round-robin (persistent grid).  A wait that
/// does not complete sets *err and the warp drains its outstanding copies
/// (again bounded) before returning.  TRANSPOSE applies the block transposed
/// (J^T v, as jvp_stored_transpose_kernel) with the same staging.
template <int C, bool HS, bool VI, int WARPS, int STAGES, bool TRANSPOSE = false, typename TS = float,
          bool SYM = false>
__global__ void __launch_bounds__(WARPS * 32) jvp_stored_tma_kernel(const float* __restrict__ du,
                                                                    const TS* __restrict__ D,
                                                                    const int32_t* __restrict__ conn,
                                                                    float* __restrict__ out_e, int64_t num_nodes,
                                                                    int64_t num_elements, int* __restrict__ err) {
  constexpr int P = 2, Q = 3, NQ = 27;
  using Shape = TangentShape<C, HS, VI, SYM>;
  // input side (interpolated direction) and output side (integrated) of the
  // block: D[out][in] for J, D^T for J^T
  constexpr bool IN_VALUE = TRANSPOSE ? HS : VI;
  constexpr bool OUT_VALUE = TRANSPOSE ? VI : HS;
  constexpr int NIN = TRANSPOSE ? Shape::rows : Shape::cols;
  constexpr int NOUT = TRANSPOSE ? Shape::cols : Shape::rows;
  constexpr int64_t ES = Shape::template stride_of<NQ, TS>;  // entries per element block
  constexpr uint32_t BYTES = uint32_t(ES * sizeof(TS));
  static_assert(BYTES % 16 == 0, "bulk copies move multiples of 16 bytes");
  extern __shared__ __align__(128) unsigned char sfx_dyn_smem[];
  TS* ring = reinterpret_cast<TS*>(sfx_dyn_smem);                                       // [WARPS][STAGES][ES]
  uint64_t* bars = reinterpret_cast<uint64_t*>(sfx_dyn_smem + size_t(WARPS) * STAGES * BYTES);  // [WARPS][STAGES]
  __shared__ float sB[Q][Q], sD[Q][Q];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x < Q * Q) {
    const int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = float(basis_table<P>().B[i][j]);
    sD[i][j] = float(basis_table<P>().D[i][j]);
  }
  TS* my_ring = ring + size_t(wid) * STAGES * ES;
  uint64_t* my_bars = bars + wid * STAGES;
  if (lane == 0) {
    for (int s = 0; s < STAGES; s++) bulk::mbar_init(&my_bars[s], 1);
    bulk::fence_mbar_init();
  }
  __syncthreads();

  const int64_t first = int64_t(blockIdx.x) * WARPS + wid;
  const int64_t step = int64_t(gridDim.x) * WARPS;
  // prologue: the first STAGES elements of this warp
  if (lane == 0) {
    for (int s = 0; s < STAGES; s++) {
      const int64_t e = first + s * step;
      if (e < num_elements) {
        bulk::mbar_arrive_expect_tx(&my_bars[s], BYTES);
        bulk::copy_g2s(my_ring + s * ES, D + e * ES, BYTES, &my_bars[s]);
      }
    }
  }
  __syncwarp();

  const bool lane_ok = lane < NQ;
  const int qi = lane_ok ? lane : NQ - 1;
  const int ix = qi % Q, iy = (qi / Q) % Q, iz = qi / (Q * Q);
  // gather pipeline: du of the current element and the node id of the next
  // one are already in registers; each iteration issues the next element's du
  // and the node id two elements ahead before computing
  int32_t node_next = 0;
  float du_cur[C];
  {
    const int32_t node0 = (lane_ok && first < num_elements) ? conn[first * NQ + qi] : 0;
#pragma unroll
    for (int c = 0; c < C; c++) du_cur[c] = (lane_ok && first < num_elements) ? du[c * num_nodes + node0] : 0.f;
    const int64_t e1 = first + step;
    node_next = (lane_ok && e1 < num_elements) ? conn[e1 * NQ + qi] : 0;
  }
  int it = 0;
  bool failed = false;
  for (int64_t e = first; e < num_elements; e += step, it++) {
    const int s = it % STAGES;
    const uint32_t parity = uint32_t(it / STAGES) & 1u;
    const int64_t e1 = e + step, e2 = e + 2 * step;
    float du_next[C];
#pragma unroll
    for (int c = 0; c < C; c++) du_next[c] = (lane_ok && e1 < num_elements) ? du[c * num_nodes + node_next] : 0.f;
    const int32_t node_after = (lane_ok && e2 < num_elements) ? conn[e2 * NQ + qi] : 0;
    // interpolate du while the tangent is in flight
    float din[NIN];
#pragma unroll
    for (int c = 0; c < C; c++) {
      float v, g0, g1, g2;
      interpolate_colloc<Q, float>(du_cur[c], 0, ix, iy, iz, sB, sD, v, g0, g1, g2);
      if constexpr (IN_VALUE) din[c] = v;
      constexpr int off = IN_VALUE ? C : 0;
      din[off + 3 * c + 0] = g0;
      din[off + 3 * c + 1] = g1;
      din[off + 3 * c + 2] = g2;
    }
    const bool ready = __all_sync(0xffffffffu, bulk::mbar_wait(&my_bars[s], parity));
    if (!ready) {
      failed = true;
      break;
    }
    const TS* Dq = my_ring + s * ES + qi;
    float dout[NOUT];
    if constexpr (std::is_same<TS, __half>::value) {
      // FP16 copy: one half2 (entries 2j, 2j + 1 of this point) per load
      const __half2* D2 = reinterpret_cast<const __half2*>(my_ring + s * ES) + qi;
#pragma unroll
      for (int r = 0; r < NOUT; r++) dout[r] = 0.f;
      apply_pairs16<Shape, TRANSPOSE, NQ>(D2, din, dout, std::make_integer_sequence<int, Shape::pairs>{});
    } else if constexpr (Shape::packed) {
#pragma unroll
      for (int r = 0; r < NOUT; r++) dout[r] = 0.f;
#pragma unroll
      for (int r = 0; r < NOUT; r++) {
#pragma unroll
        for (int k = r; k < NIN; k++) {
          const float d = tangent_to_f32(Dq[Shape::index(r, k) * NQ]);
          dout[r] += d * din[k];
          if (k != r) dout[k] += d * din[r];
        }
      }
    } else {
#pragma unroll
      for (int r = 0; r < NOUT; r++) {
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < NIN; k++)
          acc += tangent_to_f32(Dq[(TRANSPOSE ? Shape::index(k, r) : Shape::index(r, k)) * NQ]) * din[k];
        dout[r] = acc;
      }
    }
    __syncwarp();  // every lane has read stage s
    if (lane == 0) {
      const int64_t en = e + int64_t(STAGES) * step;
      if (en < num_elements) {
        bulk::fence_proxy_async_smem();
        bulk::mbar_arrive_expect_tx(&my_bars[s], BYTES);
        bulk::copy_g2s(my_ring + s * ES, D + en * ES, BYTES, &my_bars[s]);
      }
    }
    constexpr int roff = OUT_VALUE ? C : 0;
#pragma unroll
    for (int c = 0; c < C; c++) {
      const float src = OUT_VALUE ? dout[OUT_VALUE ? c : 0] : 0.f;
      const float r = integrate_colloc<Q, OUT_VALUE, true, float>(src, dout[roff + 3 * c], dout[roff + 3 * c + 1],
                                                                dout[roff + 3 * c + 2], 0, ix, iy, iz, sB, sD);
      if (lane_ok) out_e[(e * C + c) * NQ + qi] = r;
    }
    // rotate the gather pipeline (its loads had this element's work to land)
#pragma unroll
    for (int c = 0; c < C; c++) du_cur[c] = du_next[c];
    node_next = node_after;
  }
  if (failed) {
    if (lane == 0) atomicExch(err, 1);
    // drain: the copies issued for iterations it .. it + STAGES - 1
    for (int j = 0; j < STAGES; j++) {
      const int k = it + j;
      if (first + int64_t(k) * step < num_elements) (void)bulk::mbar_wait(&my_bars[k % STAGES], uint32_t(k / STAGES) & 1u);
    }
  }
}

}  // namespace kernels
}  // namespace sfx

namespace sfx {
namespace kernels {

/// Diagonal of the element Jacobians from the stored tangent, as an E-vector
/// [e][c][node]: K[(c,i)][(c,i)] = sum_q sum_{a,b} Psi_a(i,q) D[(c,a)][(c,b)](q) Psi_b(i,q)
/// with Psi_0 = phi and Psi_{1..3} = d phi / d xi_k.  Each (a, b) term is a
/// product of 1-D factors, so the sum over the points runs as three
/// sum-factorised passes (x, y, z) of 3 FMA per lane.
template <int P, int C, bool HS, bool VI, bool SYM = false>
__global__ void __launch_bounds__(128) diag_from_tangent_kernel(const double* __restrict__ D, double* __restrict__ out_e,
                                                                int64_t num_elements) {
  using Real = double;
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q * Q;
  constexpr int EPW = 32 / NQ;
  using Shape = TangentShape<C, HS, VI, SYM>;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / NQ;
  const int qi_raw = lane - sub * NQ;
  const bool slot = sub < EPW;
  const int qi = slot ? qi_raw : NQ - 1;
  const int base = slot ? sub * NQ : 0;
  const int64_t e = warp * EPW + (slot ? sub : 0);
  const bool valid = slot && e < num_elements;
  const int ix = qi % Q, iy = (qi / Q) % Q, iz = qi / (Q * Q);

  __shared__ Real sB[Q][Q], sG[Q][Q];
  if (threadIdx.x < Q * Q) {
    int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = basis_table<P>().B[i][j];
    sG[i][j] = basis_table<P>().G[i][j];
  }
  __syncthreads();
  const int64_t nq_total = num_elements * NQ;
  const int64_t gq = e * NQ + qi;

#pragma unroll
  for (int c = 0; c < C; c++) {
    Real acc_node = 0;
#pragma unroll
    for (int a = (HS ? 0 : 1); a < 4; a++) {
#pragma unroll
      for (int b = (VI ? 0 : 1); b < 4; b++) {
        const int row = (a == 0) ? c : (HS ? C : 0) + 3 * c + (a - 1);
        const int col = (b == 0) ? c : (VI ? C : 0) + 3 * c + (b - 1);
        const int ent = Shape::packed ? Shape::index(row < col ? row : col, row < col ? col : row)
                                      : Shape::index(row, col);
        Real d = valid ? D[e * Shape::template stride<NQ> + int64_t(ent) * NQ + qi] : Real(0);
        // x-pass: T1(ix', qy, qz) = sum_qx d(qx,qy,qz) fa_x(qx,ix') fb_x(qx,ix')
        Real t1 = 0;
#pragma unroll
        for (int k = 0; k < Q; k++) {
          Real fa = (a == 1) ? sG[k][ix] : sB[k][ix];
          Real fb = (b == 1) ? sG[k][ix] : sB[k][ix];
          t1 += fa * fb * shfl(d, base + k + Q * (iy + Q * iz));
        }
        Real t2 = 0;
#pragma unroll
        for (int k = 0; k < Q; k++) {
          Real fa = (a == 2) ? sG[k][iy] : sB[k][iy];
          Real fb = (b == 2) ? sG[k][iy] : sB[k][iy];
          t2 += fa * fb * shfl(t1, base + ix + Q * (k + Q * iz));
        }
        Real t3 = 0;
#pragma unroll
        for (int k = 0; k < Q; k++) {
          Real fa = (a == 3) ? sG[k][iz] : sB[k][iz];
          Real fb = (b == 3) ? sG[k][iz] : sB[k][iz];
          t3 += fa * fb * shfl(t2, base + ix + Q * (iy + Q * k));
        }
        acc_node += t3;
      }
    }
    if (valid) out_e[(e * C + c) * NQ + qi] = acc_node;
  }
}

}  // namespace kernels
}  // namespace sfx
