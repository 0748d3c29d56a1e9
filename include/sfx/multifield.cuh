// sfx — domain integrals of several trial fields (serac's
// Functional<test(trial_0, trial_1, ...)> with DependsOn<i...>,
// functional.hpp:189-317, evaluated by domain_integral_kernels.hpp:152-361).
//
// Every argument field lives on the form's node grid (H1 of the form's
// order; an H1 field of lower order is represented exactly there), with its
// own number of components.  The kernels follow the single-field ones in
// kernels.cuh (one warp per Q2 element, lane = quadrature point = node,
// sum factorisation by warp shuffles, no atomics) with three changes:
//   * every argument field is interpolated and handed to the q-function as
//     its own tuple{value, gradient}: qf(t, tuple{X, dX/dxi}, [state&,] arg0, arg1, ...);
//   * a derivative is taken with respect to one argument W (only W carries
//     dual numbers, as serac's promote_each_to_dual_when does), and the
//     stored block has rows = test outputs (source C_T, then flux 3 C_T) and
//     cols = W's inputs (values C_W, then parent gradients 3 C_W), unpacked;
//   * the transposed action integrates onto W's field (the adjoint of the
//     parameter derivative: what a parameter sensitivity needs).
#pragma once

#include <utility>

#include "sfx/kernels.cuh"

namespace sfx {
namespace kernels {

constexpr int kMaxFields = 8;

/// the component counts of a q-function's argument fields
template <int... Cs>
struct FieldList {
  static constexpr int count = sizeof...(Cs);
  static constexpr int total = (0 + ... + Cs);
  static_assert(count >= 1 && count <= 4, "one to four argument fields");
  template <int i>
  static constexpr int comps() {
    constexpr int a[] = {Cs...};
    return a[i];
  }
  template <int i>
  static constexpr int offset() {
    constexpr int a[] = {Cs...};
    int o = 0;
    for (int k = 0; k < i; k++) o += a[k];
    return o;
  }
  /// argument and component of stacked component k
  static SFX_HDI constexpr int field_of(int k) {
    constexpr int a[] = {Cs...};
    int acc = 0;
    for (int i = 0; i < count; i++) {
      if (k < acc + a[i]) return i;
      acc += a[i];
    }
    return count - 1;
  }
  static SFX_HDI constexpr int comp_of(int k) {
    constexpr int a[] = {Cs...};
    int acc = 0;
    for (int i = 0; i < count; i++) {
      if (k < acc + a[i]) return k - acc;
      acc += a[i];
    }
    return 0;
  }
};

template <typename Real>
struct MultiArgs {
  const Real* u[kMaxFields];  // the argument fields' L-vectors [comp][node]
  const Real* dir;            // direction (JVP: field W's shape) or test-space vector (transposed action)
  Real* out_e;                // E-vector [e][comp][node] (test space, or field W for the transpose)
  const int32_t* conn;
  const Real* geom;
  double* state;
  const double* params;
  int64_t num_nodes;
  int64_t num_elements;
  double t;
};

/// shape of the stored derivative with respect to one argument
template <int CT, int CW>
struct MultiTangentShape {
  static constexpr int rows = 4 * CT;
  static constexpr int cols = 4 * CW;
  template <int NQ>
  static constexpr int64_t stride = (int64_t(rows) * cols * NQ + 3) / 4 * 4;
};

namespace detail {

/// tuple{value, gradient} of argument I; argument W carries dual numbers
/// seeded on input column seed (values first, then parent gradients)
template <typename FL, int W, int I, typename Real>
SFX_HDI auto field_arg(const Real* val, const Real (*gph)[3], int seed, const Real (*Ji)[3]) {
  constexpr int C = FL::template comps<I>();
  constexpr int off = FL::template offset<I>();
  if constexpr (I == W) {
    using S = dual<Real, Real>;
    value_t<C, S> v{};
    grad_t<C, S> g{};
    const int seed_c = seed < C ? seed : (seed - C) / 3;
    const int seed_b = seed < C ? -1 : (seed - C) % 3;
#pragma unroll
    for (int c = 0; c < C; c++) {
      comp<C>(v, c) = S{val[off + c], Real(c == seed_c && seed_b < 0)};
#pragma unroll
      for (int j = 0; j < 3; j++)
        comp<C>(g, c)[j] = S{gph[off + c][j], (c == seed_c && seed_b >= 0) ? Ji[seed_b][j] : Real(0)};
    }
    return tuple{v, g};
  } else {
    value_t<C, Real> v{};
    grad_t<C, Real> g{};
#pragma unroll
    for (int c = 0; c < C; c++) {
      comp<C>(v, c) = val[off + c];
#pragma unroll
      for (int j = 0; j < 3; j++) comp<C>(g, c)[j] = gph[off + c][j];
    }
    return tuple{v, g};
  }
}

template <typename FL, int W, typename Real, std::size_t... I>
SFX_HDI auto field_args(const Real* val, const Real (*gph)[3], int seed, const Real (*Ji)[3],
                        std::index_sequence<I...>) {
  return tuple{field_arg<FL, W, int(I), Real>(val, gph, seed, Ji)...};
}

template <typename State, typename QF, typename Pos, typename Args, std::size_t... I>
SFX_HDI auto call_multi(const QF& qf, double t, const Pos& pos, State& st, const Args& args,
                        std::index_sequence<I...>) {
  if constexpr (std::is_same<State, Nothing>::value) {
    (void)st;
    return qf(t, pos, get<I>(args)...);
  } else {
    return qf(t, pos, st, get<I>(args)...);
  }
}

/// lane layout shared by the kernels of this header
template <int P>
struct Lanes {
  static constexpr int Q = P + 1;
  static constexpr int NQ = Q * Q * Q;
  static constexpr int EPW = 32 / NQ;
  int lane, sub, qi, base, ix, iy, iz;
  int64_t e;
  bool valid;
  __device__ Lanes(int64_t num_elements) {
    lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    sub = lane / NQ;
    const int qi_raw = lane - sub * NQ;
    const bool slot = sub < EPW;
    qi = slot ? qi_raw : NQ - 1;
    base = slot ? sub * NQ : 0;
    e = warp * EPW + (slot ? sub : 0);
    valid = slot && e < num_elements;
    ix = qi % Q;
    iy = (qi / Q) % Q;
    iz = qi / (Q * Q);
  }
};

template <int P, typename Real>
__device__ void load_basis(Real (*sB)[P + 1], Real (*sG)[P + 1]) {
  constexpr int Q = P + 1;
  if (threadIdx.x < Q * Q) {
    const int i = threadIdx.x / Q, j = threadIdx.x % Q;
    sB[i][j] = Real(basis_table<P>().B[i][j]);
    sG[i][j] = Real(basis_table<P>().G[i][j]);
  }
  __syncthreads();
}

}  // namespace detail

/// Residual (W < 0) or stored derivative with respect to argument W of a
/// multi-field domain integral.  Residual: E-vector [e][CT][node].
/// Derivative: D[e * stride + (row * cols + col) * NQ + q] with det(J) w and
/// the parent-space maps folded in (the derivative serac stores in
/// evaluation_kernel_impl, domain_integral_kernels.hpp:209-214).
template <int P, int CT, typename FL, int W, typename State, typename QFMaker>
__global__ void __launch_bounds__(128) multi_domain_kernel(MultiArgs<double> a, QFMaker make_qf,
                                                           double* __restrict__ D) {
  using Real = double;
  using L = detail::Lanes<P>;
  constexpr int Q = L::Q, NQ = L::NQ;
  const L ln(a.num_elements);
  __shared__ Real sB[Q][Q], sG[Q][Q];
  detail::load_basis<P>(sB, sG);
  const int64_t nq_total = a.num_elements * NQ;
  const int64_t gq = ln.e * NQ + ln.qi;
  const int32_t node = ln.valid ? a.conn[ln.e * NQ + ln.qi] : 0;

  Real Ji[3][3];
  Real dvol = 0;
  tensor<Real, 3> X{};
  tensor<Real, 3, 3> Jm{};
  if (ln.valid) {
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

  // every argument's values and physical gradients at this point
  constexpr int CTOT = FL::total;
  Real val[CTOT], gph[CTOT][3];
#pragma unroll
  for (int k = 0; k < CTOT; k++) {
    const Real U = ln.valid ? a.u[FL::field_of(k)][FL::comp_of(k) * a.num_nodes + node] : Real(0);
    Real gp[3];
    interpolate_lane<Q, Real>(U, ln.base, ln.ix, ln.iy, ln.iz, sB, sG, val[k], gp[0], gp[1], gp[2]);
#pragma unroll
    for (int j = 0; j < 3; j++) gph[k][j] = gp[0] * Ji[0][j] + gp[1] * Ji[1][j] + gp[2] * Ji[2][j];
  }
  const auto qf = make_qf(a.params + (ln.valid ? ln.e : 0) * QFMaker::nparams);
  const auto position = tuple{X, Jm};
  using Seq = std::make_index_sequence<FL::count>;
  State st0{};
  if constexpr (!std::is_same<State, Nothing>::value) {
    if (ln.valid) load_state(st0, a.state, gq, nq_total);
  }

  if constexpr (W < 0) {
    const auto args = detail::field_args<FL, -1, Real>(val, gph, -1, Ji, Seq{});
    State st = st0;
    const auto out = detail::call_multi<State>(qf, a.t, position, st, args, Seq{});
    using SrcT = std::decay_t<decltype(get<0>(out))>;
    using FluxT = std::decay_t<decltype(get<1>(out))>;
    constexpr bool HS = has_part<RESIDUAL, SrcT>();
    constexpr bool HF = has_part<RESIDUAL, FluxT>();
#pragma unroll
    for (int c = 0; c < CT; c++) {
      Real s = 0, fl[3] = {0, 0, 0};
      if constexpr (HS) s = dvol * part<RESIDUAL, Real>(source_comp<CT>(get<0>(out), c));
      if constexpr (HF) {
        auto frow = flux_row<CT>(get<1>(out), c);
        Real fp[3];
#pragma unroll
        for (int m = 0; m < 3; m++) fp[m] = part<RESIDUAL, Real>(frow[m]);
#pragma unroll
        for (int k = 0; k < 3; k++) fl[k] = dvol * (fp[0] * Ji[k][0] + fp[1] * Ji[k][1] + fp[2] * Ji[k][2]);
      }
      const Real r = integrate_lane<Q, HS, HF, Real>(s, fl[0], fl[1], fl[2], ln.base, ln.ix, ln.iy, ln.iz, sB, sG);
      if (ln.valid) a.out_e[(ln.e * CT + c) * NQ + ln.qi] = r;
    }
  } else {
    constexpr int CW = FL::template comps<W>();
    using Shape = MultiTangentShape<CT, CW>;
#pragma unroll 1
    for (int k = 0; k < Shape::cols; k++) {
      const auto args = detail::field_args<FL, W, Real>(val, gph, k, Ji, Seq{});
      State st = st0;
      const auto out = detail::call_multi<State>(qf, a.t, position, st, args, Seq{});
      using SrcT = std::decay_t<decltype(get<0>(out))>;
      using FluxT = std::decay_t<decltype(get<1>(out))>;
      Real* Dk = D + ln.e * Shape::template stride<NQ> + int64_t(k) * NQ + ln.qi;
#pragma unroll
      for (int c = 0; c < CT; c++) {
        Real s = 0, fp[3] = {0, 0, 0};
        if constexpr (has_part<JVP, SrcT>()) s = dvol * part<JVP, Real>(source_comp<CT>(get<0>(out), c));
        if constexpr (has_part<JVP, FluxT>()) {
          auto frow = flux_row<CT>(get<1>(out), c);
#pragma unroll
          for (int m = 0; m < 3; m++) fp[m] = part<JVP, Real>(frow[m]);
        }
        if (ln.valid) {
          Dk[int64_t(c) * Shape::cols * NQ] = s;
#pragma unroll
          for (int kd = 0; kd < 3; kd++)
            Dk[int64_t(CT + 3 * c + kd) * Shape::cols * NQ] =
                dvol * (fp[0] * Ji[kd][0] + fp[1] * Ji[kd][1] + fp[2] * Ji[kd][2]);
        }
      }
    }
  }
}

/// Action of the stored derivative with respect to one argument (CW
/// components) on a direction of that field: the E-vector of the test space
/// (action_of_gradient_kernel, domain_integral_kernels.hpp:277-304);
/// TRANSPOSE: the adjoint, a test-space vector mapped onto the argument's
/// field (E-vector [e][CW][node]).
template <int P, int CT, int CW, bool TRANSPOSE>
__global__ void __launch_bounds__(128) multi_jvp_kernel(MultiArgs<double> a, const double* __restrict__ D) {
  using Real = double;
  using L = detail::Lanes<P>;
  constexpr int Q = L::Q, NQ = L::NQ;
  using Shape = MultiTangentShape<CT, CW>;
  constexpr int CIN = TRANSPOSE ? CT : CW;
  constexpr int COUT = TRANSPOSE ? CW : CT;
  const L ln(a.num_elements);
  __shared__ Real sB[Q][Q], sG[Q][Q];
  detail::load_basis<P>(sB, sG);
  const int32_t node = ln.valid ? a.conn[ln.e * NQ + ln.qi] : 0;
  Real din[4 * CIN];
#pragma unroll
  for (int c = 0; c < CIN; c++) {
    const Real U = ln.valid ? a.dir[c * a.num_nodes + node] : Real(0);
    interpolate_lane<Q, Real>(U, ln.base, ln.ix, ln.iy, ln.iz, sB, sG, din[c], din[CIN + 3 * c],
                              din[CIN + 3 * c + 1], din[CIN + 3 * c + 2]);
  }
  const Real* Dq = D + (ln.valid ? ln.e * Shape::template stride<NQ> + ln.qi : 0);
  Real dout[4 * COUT];
#pragma unroll
  for (int r = 0; r < 4 * COUT; r++) {
    Real acc = 0;
#pragma unroll
    for (int k = 0; k < 4 * CIN; k++) {
      const int64_t ent = TRANSPOSE ? int64_t(k) * Shape::cols + r : int64_t(r) * Shape::cols + k;
      acc += (ln.valid ? Dq[ent * NQ] : Real(0)) * din[k];
    }
    dout[r] = acc;
  }
#pragma unroll
  for (int c = 0; c < COUT; c++) {
    const Real r = integrate_lane<Q, true, true, Real>(dout[c], dout[COUT + 3 * c], dout[COUT + 3 * c + 1],
                                                       dout[COUT + 3 * c + 2], ln.base, ln.ix, ln.iy, ln.iz, sB, sG);
    if (ln.valid) a.out_e[(ln.e * COUT + c) * NQ + ln.qi] = r;
  }
}

}  // namespace kernels
}  // namespace sfx
