// sfx — shape sensitivities for adjoint-based design.
//
// serac obtains the shape sensitivity of a quantity of interest by assembling
// dR/dp of the shape-aware residual and applying its transpose to the adjoint
// solution (SolidMechanics::computeTimestepShapeSensitivity and
// computeDualShapeSensitivity, solid_mechanics.hpp:1421-1431, 1495-1503).
// Here (dR/dp)^T lambda is formed matrix-free, element by element: for each of
// the element's 3 (p+1)^3 shape degrees of freedom, the geometry at every
// point is seeded with that basis function on dual numbers (x' = X + p +
// eps phi_j e_c, dx'/dxi likewise), the residual's derivative is integrated
// and contracted with lambda over the element's nodes (a fixed-order lane sum),
// and the lane of node j keeps the result, so each element writes one
// [3][(p+1)^3] block that the node-owner scatter sums.  The derivative of a
// quantity of interest with respect to the shape, dQ/dp, uses the same seeds
// without the integration.  Faces do the same with their (p+1)^2 nodes and the
// area weight |dx'/ds x dx'/dt| w on duals.
#pragma once

#include "sfx/boundary.cuh"
#include "sfx/kernels.cuh"
#include "sfx/qoi.cuh"

namespace sfx {
namespace kernels {

/// Reference (trilinear) position X and Jacobian dX/dxi at the Gauss point
/// (ix, iy, iz) of an element with vertices Xv [3][8]; the callers add the
/// shape field's value and parent gradient and set the dual parts per seed.
template <int Q>
SFX_HDI void reference_point_geometry(const double* Xv, int ix, int iy, int iz, double X[3], double J[3][3]) {
  const double sp[3] = {gl_point(Q, ix), gl_point(Q, iy), gl_point(Q, iz)};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    X[i] = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++) J[i][j] = 0.0;
  }
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const int b0 = v & 1, b1 = (v >> 1) & 1, b2 = (v >> 2) & 1;
    const double N0 = b0 ? sp[0] : 1.0 - sp[0], N1 = b1 ? sp[1] : 1.0 - sp[1], N2 = b2 ? sp[2] : 1.0 - sp[2];
    const double d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0, d2 = b2 ? 1.0 : -1.0;
    const double phi = N0 * N1 * N2;
    const double g[3] = {d0 * N1 * N2, N0 * d1 * N2, N0 * N1 * d2};
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double xv = Xv[i * 8 + v];
      X[i] += xv * phi;
#pragma unroll
      for (int j = 0; j < 3; j++) J[i][j] += xv * g[j];
    }
  }
}

enum { SHAPE_VJP = 0, SHAPE_QOI = 1 };

/// Domain shape sensitivities.  MODE SHAPE_VJP: out_e[e][c][j] =
/// sum over the element's residual entries (ci, i) of lambda(ci, node i)
/// dR_e(ci, i)/dp(c, j) for the residual q-function made by make_qf;
/// MODE SHAPE_QOI: out_e[e][c][j] = dQ_e/dp(c, j) for the QoI integrand
/// make_qf(nullptr).  a.u holds u; Xe [e][3][8] reference vertices; shape the
/// current shape field (nullptr = 0); lam (SHAPE_VJP) the adjoint field.
template <int P, int C, int MODE, typename State, typename QFMaker>
__global__ void __launch_bounds__(128) shape_adjoint_kernel(DomainArgs<double> a, QFMaker make_qf,
                                                            const double* __restrict__ Xe,
                                                            const double* __restrict__ shape,
                                                            const double* __restrict__ lam,
                                                            double* __restrict__ out_e) {
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

  Real uv[C], ug[C][3], lm[C];
#pragma unroll
  for (int c = 0; c < C; c++) {
    const Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    interpolate_lane<Q, Real>(U, base, ix, iy, iz, sB, sG, uv[c], ug[c][0], ug[c][1], ug[c][2]);
    lm[c] = (MODE == SHAPE_VJP && valid) ? lam[c * a.num_nodes + node] : Real(0);
  }
  // configuration x' = X + p at the point (values of the duals)
  Real X0[3], J0[3][3];
  reference_point_geometry<Q>(Xe + (valid ? e : 0) * 24, ix, iy, iz, X0, J0);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    Real pv, pg[3];
    const Real Pn = (valid && shape) ? shape[i * a.num_nodes + node] : Real(0);
    interpolate_lane<Q, Real>(Pn, base, ix, iy, iz, sB, sG, pv, pg[0], pg[1], pg[2]);
    X0[i] += pv;
#pragma unroll
    for (int j = 0; j < 3; j++) J0[i][j] = valid ? J0[i][j] + pg[j] : Real(i == j);
  }
  const Real w = gl_weight(Q, ix) * gl_weight(Q, iy) * gl_weight(Q, iz);
  const auto qf = make_qf(a.params + (valid ? e : 0) * QFMaker::nparams);
  State st0{};
  if constexpr (!std::is_same<State, Nothing>::value) {
    if (valid) load_state(st0, a.state, gq, nq_total);
  }

  Real mine[3] = {0, 0, 0};  // this lane's node: d/dp(c, node) for c = 0..2
#pragma unroll 1
  for (int j = 0; j < NQ; j++) {
    const int jx = j % Q, jy = (j / Q) % Q, jz = j / (Q * Q);
    const Real phi = sB[ix][jx] * sB[iy][jy] * sB[iz][jz];
    const Real dphi[3] = {sG[ix][jx] * sB[iy][jy] * sB[iz][jz], sB[ix][jx] * sG[iy][jy] * sB[iz][jz],
                          sB[ix][jx] * sB[iy][jy] * sG[iz][jz]};
#pragma unroll 1
    for (int cp = 0; cp < 3; cp++) {
      tensor<S, 3> xs{};
      tensor<S, 3, 3> Js{};
#pragma unroll
      for (int i = 0; i < 3; i++) {
        xs[i] = S{X0[i], (i == cp && valid) ? phi : Real(0)};
#pragma unroll
        for (int k = 0; k < 3; k++) Js[i][k] = S{J0[i][k], (i == cp && valid) ? dphi[k] : Real(0)};
      }
      const auto Jinv = inv(Js);
      const S dvol = det(Js) * w;
      value_t<C, S> qv{};
      grad_t<C, S> qg{};
#pragma unroll
      for (int c = 0; c < C; c++) {
        comp<C>(qv, c) = S{uv[c], Real(0)};
#pragma unroll
        for (int k = 0; k < 3; k++)
          comp<C>(qg, c)[k] = ug[c][0] * Jinv[0][k] + ug[c][1] * Jinv[1][k] + ug[c][2] * Jinv[2][k];
      }
      auto call = [&]() {
        if constexpr (std::is_same<State, Nothing>::value) {
          return qf(a.t, tuple{xs, Js}, tuple{qv, qg});
        } else {
          State st = st0;
          return qf(a.t, tuple{xs, Js}, st, tuple{qv, qg});
        }
      };
      const auto out = call();
      Real contrib = 0;
      if constexpr (MODE == SHAPE_QOI) {
        contrib = part<JVP, Real>(out * dvol);
      } else {
        using SrcT = std::decay_t<decltype(get<0>(out))>;
        using FluxT = std::decay_t<decltype(get<1>(out))>;
        constexpr bool HSrc = !is_zero<typename base_scalar<SrcT>::type>::value;
        constexpr bool HFlx = !is_zero<typename base_scalar<FluxT>::type>::value;
#pragma unroll
        for (int c = 0; c < C; c++) {
          Real src = 0, f[3] = {0, 0, 0};
          if constexpr (HSrc) src = part<JVP, Real>(dvol * source_comp<C>(get<0>(out), c));
          if constexpr (HFlx) {
            auto frow = flux_row<C>(get<1>(out), c);
#pragma unroll
            for (int k = 0; k < 3; k++)
              f[k] = part<JVP, Real>(dvol * (frow[0] * Jinv[k][0] + frow[1] * Jinv[k][1] + frow[2] * Jinv[k][2]));
          }
          const Real r = integrate_lane<Q, HSrc, HFlx, Real>(src, f[0], f[1], f[2], base, ix, iy, iz, sB, sG);
          contrib += r * lm[c];
        }
      }
      const Real total = segment_sum<NQ, Real>(valid ? contrib : Real(0), base);
      if (qi_raw == j) {  // constant indices keep mine[] in registers
        if (cp == 0) mine[0] = total;
        else if (cp == 1) mine[1] = total;
        else mine[2] = total;
      }
    }
  }
  if (valid) {
#pragma unroll
    for (int cp = 0; cp < 3; cp++) out_e[(e * 3 + cp) * NQ + qi] = mine[cp];
  }
}

/// Face shape sensitivities (as shape_adjoint_kernel, over the (p+1)^2 nodes
/// of each face): SHAPE_VJP contracts the face residual's derivative with
/// lambda, SHAPE_QOI differentiates the face QoI integrand.  out_e [f][3][node].
template <int P, int C, int MODE, typename QF>
__global__ void __launch_bounds__(128) face_shape_adjoint_kernel(FaceArgs<double> a, QF qf,
                                                                 const double* __restrict__ Xf,
                                                                 const double* __restrict__ shape,
                                                                 const double* __restrict__ lam) {
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

  Real uv[C], us[C], ut[C], lm[C];
#pragma unroll
  for (int c = 0; c < C; c++) {
    const Real U = valid ? a.u[c * a.num_nodes + node] : Real(0);
    face_interpolate<Q, Real>(U, base, ix, iy, sB, sG, uv[c], us[c], ut[c]);
    lm[c] = (MODE == SHAPE_VJP && valid) ? lam[c * a.num_nodes + node] : Real(0);
  }
  // x' = X + p on the face (values)
  Real X0[3], J0[3][2];
  {
    const Real sp[2] = {gl_point(Q, ix), gl_point(Q, iy)};
    const Real* Xv = Xf + (valid ? f : 0) * 12;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      X0[i] = 0;
      J0[i][0] = 0;
      J0[i][1] = 0;
    }
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const int b0 = v & 1, b1 = (v >> 1) & 1;
      const Real N0 = b0 ? sp[0] : 1.0 - sp[0], N1 = b1 ? sp[1] : 1.0 - sp[1];
      const Real d0 = b0 ? 1.0 : -1.0, d1 = b1 ? 1.0 : -1.0;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const Real xv = Xv[i * 4 + v];
        X0[i] += xv * N0 * N1;
        J0[i][0] += xv * d0 * N1;
        J0[i][1] += xv * N0 * d1;
      }
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
      Real pv, ps, pt;
      const Real Pn = (valid && shape) ? shape[i * a.num_nodes + node] : Real(0);
      face_interpolate<Q, Real>(Pn, base, ix, iy, sB, sG, pv, ps, pt);
      X0[i] += pv;
      J0[i][0] += ps;
      J0[i][1] += pt;
    }
    if (!valid) {
#pragma unroll
      for (int i = 0; i < 3; i++) {
        J0[i][0] = Real(i == 0);
        J0[i][1] = Real(i == 1);
      }
    }
  }
  const Real w = gl_weight(Q, ix) * gl_weight(Q, iy);

  Real mine[3] = {0, 0, 0};
#pragma unroll 1
  for (int j = 0; j < NQ; j++) {
    const int jx = j % Q, jy = j / Q;
    const Real phi = sB[ix][jx] * sB[iy][jy];
    const Real dphi[2] = {sG[ix][jx] * sB[iy][jy], sB[ix][jx] * sG[iy][jy]};
#pragma unroll 1
    for (int cp = 0; cp < 3; cp++) {
      tensor<S, 3> xs{};
      tensor<S, 3, 2> Js{};
#pragma unroll
      for (int i = 0; i < 3; i++) {
        xs[i] = S{X0[i], (i == cp && valid) ? phi : Real(0)};
        Js[i][0] = S{J0[i][0], (i == cp && valid) ? dphi[0] : Real(0)};
        Js[i][1] = S{J0[i][1], (i == cp && valid) ? dphi[1] : Real(0)};
      }
      const S n0 = Js[1][0] * Js[2][1] - Js[2][0] * Js[1][1];
      const S n1 = Js[2][0] * Js[0][1] - Js[0][0] * Js[2][1];
      const S n2 = Js[0][0] * Js[1][1] - Js[1][0] * Js[0][1];
      const S n2sum = n0 * n0 + n1 * n1 + n2 * n2;
      const Real nrm = ::sqrt(n2sum.value);
      const S weight = S{nrm * w, nrm > 0 ? 0.5 * n2sum.gradient / nrm * w : Real(0)};
      fvalue_t<C, S> qv{};
      fgrad_t<C, S> qg{};
#pragma unroll
      for (int c = 0; c < C; c++) {
        comp<C>(qv, c) = S{uv[c], Real(0)};
        comp<C>(qg, c)[0] = S{us[c], Real(0)};
        comp<C>(qg, c)[1] = S{ut[c], Real(0)};
      }
      const auto out = qf(a.t, tuple{xs, Js}, tuple{qv, qg});
      Real contrib = 0;
      if constexpr (MODE == SHAPE_QOI) {
        contrib = part<JVP, Real>(weight * out);
      } else {
        using OutT = std::decay_t<decltype(out)>;
        constexpr bool HS = !is_zero<typename base_scalar<OutT>::type>::value;
#pragma unroll
        for (int c = 0; c < C; c++) {
          Real sv = 0;
          if constexpr (HS) sv = part<JVP, Real>(weight * source_comp<C>(out, c));
          contrib += face_integrate<Q, Real>(sv, base, ix, iy, sB) * lm[c];
        }
      }
      const Real total = segment_sum<NQ, Real>(valid ? contrib : Real(0), base);
      if (qi_raw == j) {  // constant indices keep mine[] in registers
        if (cp == 0) mine[0] = total;
        else if (cp == 1) mine[1] = total;
        else mine[2] = total;
      }
    }
  }
  if (valid) {
#pragma unroll
    for (int cp = 0; cp < 3; cp++) a.out_e[(f * 3 + cp) * NQ + qi] = mine[cp];
  }
}

}  // namespace kernels
}  // namespace sfx
