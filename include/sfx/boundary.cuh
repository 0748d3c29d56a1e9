// sfx — boundary-face kernels (quadrilateral faces of hexahedral meshes).
//
// serac's boundary integrals (boundary_integral_kernels.hpp:112-325) evaluate
// the q-function at the Gauss points of each face with the trial values and
// their derivatives with respect to the two face coordinates, multiply the
// returned value by |dX/ds x dX/dt| and integrate it against the face basis
// (a source term only).  Here the (p+1)^2 points of a face sit on
// consecutive lanes of a warp (three Q2 faces or eight Q1 faces per warp) and
// the 2-D sum factorisation runs with warp shuffles, like the hexahedron
// kernels.
#pragma once

#include "sfx/kernels.cuh"

namespace sfx {
namespace kernels {

/// Face geometric factors, structure-of-arrays over all face points:
///   k = 0..2 X, k = 3..8 J (row-major [x][s]), k = 9 |J_s x J_t| w_q
constexpr int FGEOM_STRIDE = 10;

template <typename Real>
struct FaceArgs {
  const Real* u;
  const Real* du;
  Real* out_e;               // [f][c][node]
  const int32_t* fconn;      // [f][(p+1)^2]
  const double* fgeom;       // FGEOM_STRIDE x nq_total
  int64_t num_nodes;
  int64_t num_faces;
  double t;
};

template <int C, typename T>
using fvalue_t = std::conditional_t<C == 1, T, tensor<T, C>>;
template <int C, typename T>
using fgrad_t = std::conditional_t<C == 1, tensor<T, 2>, tensor<T, C, 2>>;

template <int Q, typename Real>
SFX_HDI void face_interpolate(Real U, int base, int ix, int iy, const Real (*B)[Q], const Real (*G)[Q], Real& v,
                              Real& gs, Real& gt) {
  Real A0 = 0, A1 = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    Real x = shfl(U, base + k + Q * iy);
    A0 += B[ix][k] * x;
    A1 += G[ix][k] * x;
  }
  Real a = 0, b = 0, c = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    int src = base + ix + Q * k;
    Real a0 = shfl(A0, src), a1 = shfl(A1, src);
    a += B[iy][k] * a0;
    b += B[iy][k] * a1;
    c += G[iy][k] * a0;
  }
  v = a;
  gs = b;
  gt = c;
}

template <int Q, typename Real>
SFX_HDI Real face_integrate(Real s, int base, int ix, int iy, const Real (*B)[Q]) {
  Real a = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) a += B[k][ix] * shfl(s, base + k + Q * iy);
  Real r = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) r += B[k][iy] * shfl(a, base + ix + Q * k);
  return r;
}

/// RESIDUAL or JVP (directional duals) over the faces of one boundary integral.
template <int P, int C, int MODE, typename Real, typename QF>
__global__ void __launch_bounds__(128) face_kernel(FaceArgs<Real> a, QF qf) {
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

  using S = std::conditional_t<MODE == JVP, dual<Real, Real>, Real>;
  fvalue_t<C, S> qv{};
  fgrad_t<C, S> qg{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    Real v, gs, gt;
    face_interpolate<Q, Real>(U, base, ix, iy, sB, sG, v, gs, gt);
    if constexpr (MODE == JVP) {
      Real dU = valid ? a.du[c * a.num_nodes + node] : Real(0);
      Real dv, dgs, dgt;
      face_interpolate<Q, Real>(dU, base, ix, iy, sB, sG, dv, dgs, dgt);
      comp<C>(qv, c) = S{v, dv};
      comp<C>(qg, c)[0] = S{gs, dgs};
      comp<C>(qg, c)[1] = S{gt, dgt};
    } else {
      comp<C>(qv, c) = v;
      comp<C>(qg, c)[0] = gs;
      comp<C>(qg, c)[1] = gt;
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
    scale = Real(g[9 * nq_total]);
  }
  auto out = qf(a.t, tuple{X, J}, tuple{qv, qg});
  using OutT = std::decay_t<decltype(out)>;
  constexpr bool HS = has_part<MODE, OutT>();
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real s = 0;
    if constexpr (HS) s = scale * part<MODE, Real>(source_comp<C>(out, c));
    Real r = face_integrate<Q, Real>(s, base, ix, iy, sB);
    if (valid) a.out_e[(f * C + c) * NQ + qi] = r;
  }
}

/// Transpose of face_interpolate applied to (value, d/ds, d/dt) data at the
/// points: r(node) = sum over points of B s + G_s fs + G_t ft, for this lane's
/// node.
template <int Q, typename Real>
SFX_HDI Real face_integrate_full(Real s, Real fs, Real ft, int base, int ix, int iy, const Real (*B)[Q],
                                 const Real (*G)[Q]) {
  Real a = 0, b = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    const int src = base + k + Q * iy;
    a += B[k][ix] * shfl(s, src) + G[k][ix] * shfl(fs, src);
    b += B[k][ix] * shfl(ft, src);
  }
  Real r = 0;
#pragma unroll
  for (int k = 0; k < Q; k++) {
    const int src = base + ix + Q * k;
    r += B[k][iy] * shfl(a, src) + G[k][iy] * shfl(b, src);
  }
  return r;
}

/// Transposed Jacobian action of a boundary integral, dr = J^T v at the
/// linearisation point a.u (a.du holds v).  Per point, the derivative of the
/// q-function output (times the area weight) with respect to each trial
/// component's value and surface derivatives is formed by directional duals
/// (as in face_matrix_kernel); its transpose is applied to v at the point and
/// integrated against the face basis and its surface derivatives.
template <int P, int C, typename Real, typename QF>
__global__ void __launch_bounds__(128) face_jvp_transpose_kernel(FaceArgs<Real> a, QF qf) {
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
    sB[i][j] = Real(basis_table<P>().B[i][j]);
    sG[i][j] = Real(basis_table<P>().G[i][j]);
  }
  __syncthreads();
  const int64_t nq_total = a.num_faces * NQ;
  const int64_t gq = f * NQ + qi;
  const int32_t node = valid ? a.fconn[f * NQ + qi] : 0;

  Real uv[C], ugs[C], ugt[C], vq[C];
#pragma unroll
  for (int c = 0; c < C; c++) {
    const Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    face_interpolate<Q, Real>(U, base, ix, iy, sB, sG, uv[c], ugs[c], ugt[c]);
    const Real V = valid ? a.du[c * a.num_nodes + node] : Real(0);
    Real vs, vt;
    face_interpolate<Q, Real>(V, base, ix, iy, sB, sG, vq[c], vs, vt);
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
    scale = Real(g[9 * nq_total]);
  }
  using S = dual<Real, Real>;
#pragma unroll 1
  for (int cj = 0; cj < C; cj++) {
    Real w[3];  // sum over ci of v_ci d(out_ci)/d(value, d/ds, d/dt of component cj)
#pragma unroll
    for (int b = 0; b < 3; b++) {
      fvalue_t<C, S> qv{};
      fgrad_t<C, S> qg{};
#pragma unroll
      for (int c = 0; c < C; c++) {
        comp<C>(qv, c) = S{uv[c], Real(c == cj && b == 0)};
        comp<C>(qg, c)[0] = S{ugs[c], Real(c == cj && b == 1)};
        comp<C>(qg, c)[1] = S{ugt[c], Real(c == cj && b == 2)};
      }
      auto out = qf(a.t, tuple{X, J}, tuple{qv, qg});
      using OutT = std::decay_t<decltype(out)>;
      Real acc = 0;
#pragma unroll
      for (int ci = 0; ci < C; ci++) {
        if constexpr (has_part<JVP, OutT>()) acc += part<JVP, Real>(source_comp<C>(out, ci)) * vq[ci];
      }
      w[b] = scale * acc;
    }
    const Real r = face_integrate_full<Q, Real>(w[0], w[1], w[2], base, ix, iy, sB, sG);
    if (valid) a.out_e[(f * C + cj) * NQ + qi] = r;
  }
}

/// Derivative of a shape-aware boundary integral with respect to the shape
/// displacement, applied to dp (serac's ShapeAwareBoundaryIntegrandWrapper,
/// shape_aware_functional.hpp:475-498, differentiated with respect to the
/// shape): x' = X + p + eps dp and dx'/d(s,t) = J + dp/d(s,t) + eps d(dp)/d(s,t)
/// on dual numbers, so the q-function value and the area weight
/// |dx'/ds x dx'/dt| w carry the directional derivative; its derivative part
/// is integrated into out_e [f][c][node].  Xf: [f][3][4] face vertices,
/// shape (nullptr = 0) and dshape: byNODES 3-component fields of order P.
template <int P, int C, typename QF>
__global__ void __launch_bounds__(128) face_shape_jvp_kernel(FaceArgs<double> a, QF qf,
                                                             const double* __restrict__ Xf,
                                                             const double* __restrict__ shape,
                                                             const double* __restrict__ dshape) {
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
  const int32_t node = valid ? a.fconn[f * NQ + qi] : 0;

  fvalue_t<C, S> qv{};
  fgrad_t<C, S> qg{};
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    Real v, gs, gt;
    face_interpolate<Q, Real>(U, base, ix, iy, sB, sG, v, gs, gt);
    comp<C>(qv, c) = S{v, Real(0)};
    comp<C>(qg, c)[0] = S{gs, Real(0)};
    comp<C>(qg, c)[1] = S{gt, Real(0)};
  }
  // shape field and direction at the point
  tensor<S, 3> X{};
  tensor<S, 3, 2> J{};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    Real pv, ps, pt, dv, ds, dt;
    const Real Pn = (valid && shape) ? shape[i * a.num_nodes + node] : Real(0);
    const Real dPn = valid ? dshape[i * a.num_nodes + node] : Real(0);
    face_interpolate<Q, Real>(Pn, base, ix, iy, sB, sG, pv, ps, pt);
    face_interpolate<Q, Real>(dPn, base, ix, iy, sB, sG, dv, ds, dt);
    X[i] = S{pv, dv};
    J[i][0] = S{ps, ds};
    J[i][1] = S{pt, dt};
  }
  // reference (bilinear) face geometry
  const Real sp[2] = {gl_point(Q, ix), gl_point(Q, iy)};
  const Real w = gl_weight(Q, ix) * gl_weight(Q, iy);
  const Real* Xv = Xf + (valid ? f : 0) * 12;
#pragma unroll
  for (int v = 0; v < 4; v++) {
    const int b0 = v & 1, b1 = (v >> 1) & 1;
    const Real N0 = b0 ? sp[0] : 1.0 - sp[0], N1 = b1 ? sp[1] : 1.0 - sp[1];
    const Real d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const Real xv = Xv[i * 4 + v];
      X[i].value += xv * N0 * N1;
      J[i][0].value += xv * d0 * N1;
      J[i][1].value += xv * N0 * d1;
    }
  }
  const S n0 = J[1][0] * J[2][1] - J[2][0] * J[1][1];
  const S n1 = J[2][0] * J[0][1] - J[0][0] * J[2][1];
  const S n2 = J[0][0] * J[1][1] - J[1][0] * J[0][1];
  const S n2sum = n0 * n0 + n1 * n1 + n2 * n2;
  const Real nrm = ::sqrt(n2sum.value);
  const S weight = S{nrm * w, valid && nrm > 0 ? 0.5 * n2sum.gradient / nrm * w : Real(0)};
  auto out = qf(a.t, tuple{X, J}, tuple{qv, qg});
  using OutT = std::decay_t<decltype(out)>;
  constexpr bool HS = !is_zero<typename base_scalar<OutT>::type>::value;
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real s = 0;
    if constexpr (HS) s = part<JVP, Real>(weight * source_comp<C>(out, c));
    Real r = face_integrate<Q, Real>(s, base, ix, iy, sB);
    if (valid) a.out_e[(f * C + c) * NQ + qi] = r;
  }
}

/// Face element matrices K[f][trial vdof][test vdof] (as the domain ones),
/// by directional duals seeded on each parent-space input of each trial
/// component, then one face integration per trial node.
template <int P, int C, typename QF>
__global__ void __launch_bounds__(128) face_matrix_kernel(FaceArgs<double> a, QF qf) {
  using Real = double;
  constexpr int Q = P + 1;
  constexpr int NQ = Q * Q;
  constexpr int FPW = 32 / NQ;
  constexpr int NDOF = C * NQ;
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

  Real uv[C], ugs[C], ugt[C];
#pragma unroll
  for (int c = 0; c < C; c++) {
    Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    face_interpolate<Q, Real>(U, base, ix, iy, sB, sG, uv[c], ugs[c], ugt[c]);
  }
  tensor<Real, 3> X{};
  tensor<Real, 3, 2> J{};
  Real scale = 0;
  if (valid) {
    const double* g = a.fgeom + gq;
#pragma unroll
    for (int k = 0; k < 3; k++) X[k] = g[k * nq_total];
#pragma unroll
    for (int k = 0; k < 6; k++) J[k / 2][k % 2] = g[(3 + k) * nq_total];
    scale = g[9 * nq_total];
  }
  using S = dual<Real, Real>;
#pragma unroll 1
  for (int cj = 0; cj < C; cj++) {
    Real Dv[C][3];  // d out_ci / d (value, d/ds, d/dt) of component cj
#pragma unroll
    for (int b = 0; b < 3; b++) {
      fvalue_t<C, S> qv{};
      fgrad_t<C, S> qg{};
#pragma unroll
      for (int c = 0; c < C; c++) {
        comp<C>(qv, c) = S{uv[c], Real(c == cj && b == 0)};
        comp<C>(qg, c)[0] = S{ugs[c], Real(c == cj && b == 1)};
        comp<C>(qg, c)[1] = S{ugt[c], Real(c == cj && b == 2)};
      }
      auto out = qf(a.t, tuple{X, J}, tuple{qv, qg});
      using OutT = std::decay_t<decltype(out)>;
#pragma unroll
      for (int ci = 0; ci < C; ci++) {
        if constexpr (has_part<JVP, OutT>()) Dv[ci][b] = scale * part<JVP, Real>(source_comp<C>(out, ci));
        else Dv[ci][b] = 0;
      }
    }
#pragma unroll 1
    for (int j = 0; j < NQ; j++) {
      const int jx = j % Q, jy = j / Q;
      const Real psi0 = sB[ix][jx] * sB[iy][jy], psi1 = sG[ix][jx] * sB[iy][jy], psi2 = sB[ix][jx] * sG[iy][jy];
      Real* col = a.out_e + (f * NDOF + (cj * NQ + j)) * int64_t(NDOF);
#pragma unroll
      for (int ci = 0; ci < C; ci++) {
        Real s = Dv[ci][0] * psi0 + Dv[ci][1] * psi1 + Dv[ci][2] * psi2;
        Real r = face_integrate<Q, Real>(s, base, ix, iy, sB);
        if (valid) col[ci * NQ + qi] = r;
      }
    }
  }
}

/// Face geometric factors of bilinear quadrilaterals (geometric_factors.cpp:140-220).
/// Xf: [f][3][4] corner coordinates in (s, t) lexicographic order.
template <int Q>
__global__ void face_geometry_kernel(const double* __restrict__ Xf, double* __restrict__ g, int64_t nf) {
  constexpr int NQ = Q * Q;
  const int64_t nqt = nf * NQ;
  int64_t gq = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gq >= nqt) return;
  int64_t f = gq / NQ;
  int q = int(gq - f * NQ);
  int qx = q % Q, qy = q / Q;
  double s[2] = {gl_point(Q, qx), gl_point(Q, qy)};
  double w = gl_weight(Q, qx) * gl_weight(Q, qy);
  const double* X = Xf + f * 12;
  double x[3] = {0, 0, 0}, J[3][2] = {};
  for (int v = 0; v < 4; v++) {
    int b0 = v & 1, b1 = (v >> 1) & 1;
    double N0 = b0 ? s[0] : 1.0 - s[0], N1 = b1 ? s[1] : 1.0 - s[1];
    double d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0;
    for (int i = 0; i < 3; i++) {
      double xv = X[i * 4 + v];
      x[i] += xv * N0 * N1;
      J[i][0] += xv * d0 * N1;
      J[i][1] += xv * N0 * d1;
    }
  }
  double n0 = J[1][0] * J[2][1] - J[2][0] * J[1][1];
  double n1 = J[2][0] * J[0][1] - J[0][0] * J[2][1];
  double n2 = J[0][0] * J[1][1] - J[1][0] * J[0][1];
  double vals[FGEOM_STRIDE] = {x[0], x[1], x[2], J[0][0], J[0][1], J[1][0], J[1][1], J[2][0], J[2][1],
                               ::sqrt(n0 * n0 + n1 * n1 + n2 * n2) * w};
  for (int k = 0; k < FGEOM_STRIDE; k++) g[k * nqt + gq] = vals[k];
}

/// Face geometry of the shape-displaced configuration: x' = X + p,
/// dx'/dxi = dX/dxi + dp/dxi and weight |cross(dx'/dxi)| w, which is serac's
/// boundary area correction (shape_aware_functional.hpp:155-172) applied to
/// the reference weight.  p: 3-component order-P field on the node grid
/// (byNODES), gathered through the face connectivity [f][(P+1)^2].
template <int P>
__global__ void face_geometry_shape_kernel(const double* __restrict__ Xf, const int32_t* __restrict__ fconn,
                                           const double* __restrict__ shape, int64_t num_nodes,
                                           double* __restrict__ g, int64_t nf) {
  constexpr int Q = P + 1, NQ = Q * Q, N1 = P + 1, NPF = N1 * N1;
  const int64_t nqt = nf * NQ;
  int64_t gq = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gq >= nqt) return;
  int64_t f = gq / NQ;
  int q = int(gq - f * NQ);
  int qx = q % Q, qy = q / Q;
  double s[2] = {gl_point(Q, qx), gl_point(Q, qy)};
  double w = gl_weight(Q, qx) * gl_weight(Q, qy);
  const double* X = Xf + f * 12;
  double x[3] = {0, 0, 0}, J[3][2] = {};
  for (int v = 0; v < 4; v++) {
    int b0 = v & 1, b1 = (v >> 1) & 1;
    double N0 = b0 ? s[0] : 1.0 - s[0], N1v = b1 ? s[1] : 1.0 - s[1];
    double d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0;
    for (int i = 0; i < 3; i++) {
      double xv = X[i * 4 + v];
      x[i] += xv * N0 * N1v;
      J[i][0] += xv * d0 * N1v;
      J[i][1] += xv * N0 * d1;
    }
  }
  const auto& T = basis_table<P>();
  const int32_t* cf = fconn + f * NPF;
  for (int a = 0; a < NPF; a++) {
    const int as = a % N1, at = a / N1;
    const double phi = T.B[qx][as] * T.B[qy][at];
    const double gs = T.G[qx][as] * T.B[qy][at], gt = T.B[qx][as] * T.G[qy][at];
    const int64_t node = cf[a];
    for (int i = 0; i < 3; i++) {
      const double pv = shape[i * num_nodes + node];
      x[i] += pv * phi;
      J[i][0] += pv * gs;
      J[i][1] += pv * gt;
    }
  }
  double n0 = J[1][0] * J[2][1] - J[2][0] * J[1][1];
  double n1 = J[2][0] * J[0][1] - J[0][0] * J[2][1];
  double n2 = J[0][0] * J[1][1] - J[1][0] * J[0][1];
  double vals[FGEOM_STRIDE] = {x[0], x[1], x[2], J[0][0], J[0][1], J[1][0], J[1][1], J[2][0], J[2][1],
                               ::sqrt(n0 * n0 + n1 * n1 + n2 * n2) * w};
  for (int k = 0; k < FGEOM_STRIDE; k++) g[k * nqt + gq] = vals[k];
}

/// out[c * N + node_ids[i]] += sum over the compact face-node entry list (in
/// face order) of E[(f * C + c) * NPF + local].  One thread per face node.
template <int C, int NPF, typename Real>
__global__ void face_scatter_kernel(const Real* __restrict__ E, const int32_t* __restrict__ node_ptr,
                                    const int32_t* __restrict__ node_ids, const int32_t* __restrict__ node_ent,
                                    Real* __restrict__ out, int64_t num_face_nodes, int64_t num_nodes) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= num_face_nodes) return;
  const int64_t n = node_ids[i];
  Real acc[C];
#pragma unroll
  for (int c = 0; c < C; c++) acc[c] = 0.0;
  for (int32_t k = node_ptr[i]; k < node_ptr[i + 1]; k++) {
    const int32_t ent = node_ent[k];
    const int64_t f = ent / NPF;
    const int loc = ent - int(f) * NPF;
#pragma unroll
    for (int c = 0; c < C; c++) acc[c] += E[(f * C + c) * NPF + loc];
  }
#pragma unroll
  for (int c = 0; c < C; c++) out[c * num_nodes + n] += acc[c];
}

/// diag[c * N + node] += sum over the node's faces of K[f][(c,a)][(c,a)]
template <int C, int NPF>
__global__ void face_diag_kernel(const int32_t* __restrict__ node_ptr, const int32_t* __restrict__ node_ids,
                                 const int32_t* __restrict__ node_ent, const double* __restrict__ Kf,
                                 double* __restrict__ diag, int64_t num_face_nodes, int64_t num_nodes) {
  constexpr int NDOF = C * NPF;
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= num_face_nodes) return;
  const int64_t n = node_ids[i];
  for (int c = 0; c < C; c++) {
    double acc = 0.0;
    for (int32_t k = node_ptr[i]; k < node_ptr[i + 1]; k++) {
      const int32_t ent = node_ent[k];
      const int64_t f = ent / NPF;
      const int a = ent - int(f) * NPF;
      const int64_t d = c * NPF + a;
      acc += Kf[f * NDOF * NDOF + d * NDOF + d];
    }
    diag[c * num_nodes + n] += acc;
  }
}

/// CSR values of the face contributions: one thread per (component, face
/// node) row adds its faces' element-matrix entries in face order.
template <int P, int C, typename Graph>
__global__ void face_csr_kernel(Graph g, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ fconn,
                                const int32_t* __restrict__ node_ptr, const int32_t* __restrict__ node_ids,
                                const int32_t* __restrict__ node_ent, const double* __restrict__ Kf,
                                double* __restrict__ values, int64_t num_face_nodes) {
  constexpr int NPF = (P + 1) * (P + 1);
  constexpr int NDOF = C * NPF;
  const int64_t nn = g.num_nodes();
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= num_face_nodes * C) return;
  const int ci = int(t / num_face_nodes);
  const int64_t i = t - ci * num_face_nodes;
  const int64_t node = node_ids[i];
  const int64_t r = ci * nn + node;
  const auto grow = g.row(node);
  const int64_t scalar_len = grow.len;
  double* row = values + row_ptr[r];
  for (int32_t k = node_ptr[i]; k < node_ptr[i + 1]; k++) {
    const int32_t ent = node_ent[k];
    const int64_t f = ent / NPF;
    const int a = ent - int(f) * NPF;
    const double* Kcol = Kf + f * NDOF * NDOF + (ci * NPF + a);
    for (int b = 0; b < NPF; b++) {
      const int64_t pos = g.pos(grow, fconn[f * NPF + b]);
#pragma unroll
      for (int cj = 0; cj < C; cj++) row[cj * scalar_len + pos] += Kcol[int64_t(cj * NPF + b) * NDOF];
    }
  }
}

}  // namespace kernels
}  // namespace sfx
