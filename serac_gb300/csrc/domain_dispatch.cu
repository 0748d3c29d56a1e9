// Instantiates the fused domain kernels for the material library and
// dispatches on (order, material, mode, precision).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <type_traits>

#include "dispatch.hpp"
#include "form.hpp"
#include "sfx/kernels.cuh"
#include "sfx/materials.hpp"
#include "sfx/sensitivity.cuh"

namespace sfx_impl {
namespace {

using namespace sfx;
using J2 = solid_mechanics::J2SmallStrain<solid_mechanics::LinearHardening>;

// symmetric_tangent: the stored derivative block is symmetric (the flux is
// the gradient of a potential in the trial gradient), so it is stored packed
struct HeatMaker {
  static constexpr int nparams = 2;
  static constexpr bool value_input = false;
  static constexpr bool symmetric_tangent = true;
  SFX_HD heat_transfer::HeatIntegrand operator()(const double* p) const {
    heat_transfer::HeatIntegrand q{};
    q.material.conductivity = p[0];
    q.source = p[1];
    return q;
  }
};
struct NonlinearHeatMaker {
  static constexpr int nparams = 3;
  static constexpr bool value_input = true;
  SFX_HD heat_transfer::NonlinearHeatIntegrand operator()(const double* p) const {
    return heat_transfer::NonlinearHeatIntegrand{p[0], p[1], p[2]};
  }
};
struct NeoHookeanMaker {
  static constexpr int nparams = 2;
  static constexpr bool value_input = false;
  static constexpr bool symmetric_tangent = true;  // first Piola stress = dW/dF
  SFX_HD solid_mechanics::MaterialStressFunctor<solid_mechanics::NeoHookean, true> operator()(const double* p) const {
    return {solid_mechanics::NeoHookean{1.0, p[0], p[1]}};
  }
};
struct J2Maker {
  static constexpr int nparams = 4;
  static constexpr bool value_input = false;
  static constexpr bool symmetric_tangent = true;  // associative flow, linear isotropic hardening
  SFX_HD solid_mechanics::MaterialStressFunctor<J2, false> operator()(const double* p) const {
    J2 m{};
    m.E = p[0];
    m.nu = p[1];
    m.hardening = solid_mechanics::LinearHardening{p[2], p[3]};
    m.Hk = 0.0;
    m.density = 1.0;
    return {m};
  }
};
struct ThermalTestMaker {
  static constexpr int nparams = 0;
  static constexpr bool value_input = true;
  SFX_HD test_models::ThermalModel operator()(const double*) const { return {}; }
};
struct ElasticTestMaker {
  static constexpr int nparams = 0;
  static constexpr bool value_input = true;
  SFX_HD test_models::ElasticModel operator()(const double*) const { return {}; }
};

// Maker::symmetric_tangent where declared, false otherwise
template <typename M, typename = void>
struct sym_of : std::false_type {};
template <typename M>
struct sym_of<M, std::void_t<decltype(M::symmetric_tangent)>> : std::bool_constant<M::symmetric_tangent> {};

// Calls fn.template operator()<C, State, Maker>() for the form's material.
template <typename Fn>
int visit_material(int material, Fn&& fn) {
  switch (material) {
    case SFX_MAT_HEAT: return fn.template operator()<1, Nothing, HeatMaker>();
    case SFX_MAT_NONLINEAR_HEAT: return fn.template operator()<1, Nothing, NonlinearHeatMaker>();
    case SFX_MAT_THERMAL_TEST: return fn.template operator()<1, Nothing, ThermalTestMaker>();
    case SFX_MAT_ELASTIC_TEST: return fn.template operator()<3, Nothing, ElasticTestMaker>();
    case SFX_MAT_NEOHOOKEAN: return fn.template operator()<3, Empty, NeoHookeanMaker>();
    case SFX_MAT_J2: return fn.template operator()<3, J2::State, J2Maker>();
  }
  return fail(SFX_ERR_UNSUPPORTED, "unknown material");
}

template <int P, int C, int MODE, typename Real, typename State, typename Maker>
int launch(const sfx_form_s& f, const DomainIntegral& di, const Real* u, const Real* du, Real* E, const Real* geom,
           double t, cudaStream_t s) {
  constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
  constexpr int EPW = 32 / NQ;
  if (f.ne == 0) return SFX_OK;
  kernels::DomainArgs<Real> a{u, du, E, f.conn.p, geom, di.state.p, di.params.p, f.nnodes, f.ne, t};
  int64_t warps = (f.ne + EPW - 1) / EPW;
  int64_t blocks = (warps * 32 + 127) / 128;
  kernels::domain_kernel<P, C, MODE, Real, State, Maker><<<unsigned(blocks), 128, 0, s>>>(a, Maker{});
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("domain kernel launch: ") + cudaGetErrorString(err));
  return SFX_OK;
}

template <int MODE, typename Real, int P>
int dispatch_p(const sfx_form_s& f, const DomainIntegral& di, const Real* u, const Real* du, Real* E,
               const Real* geom, double t, cudaStream_t s) {
  switch (di.material) {
    case SFX_MAT_HEAT: return launch<P, 1, MODE, Real, Nothing, HeatMaker>(f, di, u, du, E, geom, t, s);
    case SFX_MAT_NONLINEAR_HEAT:
      return launch<P, 1, MODE, Real, Nothing, NonlinearHeatMaker>(f, di, u, du, E, geom, t, s);
    case SFX_MAT_THERMAL_TEST: return launch<P, 1, MODE, Real, Nothing, ThermalTestMaker>(f, di, u, du, E, geom, t, s);
    case SFX_MAT_ELASTIC_TEST: return launch<P, 3, MODE, Real, Nothing, ElasticTestMaker>(f, di, u, du, E, geom, t, s);
    case SFX_MAT_NEOHOOKEAN: return launch<P, 3, MODE, Real, Empty, NeoHookeanMaker>(f, di, u, du, E, geom, t, s);
    case SFX_MAT_J2: return launch<P, 3, MODE, Real, J2::State, J2Maker>(f, di, u, du, E, geom, t, s);
  }
  return fail(SFX_ERR_UNSUPPORTED, "unknown material");
}

template <int MODE, typename Real>
int dispatch(const sfx_form_s& f, const DomainIntegral& di, const Real* u, const Real* du, Real* E, const Real* geom,
             double t, cudaStream_t s) {
  if (f.p == 1) return dispatch_p<MODE, Real, 1>(f, di, u, du, E, geom, t, s);
  if (f.p == 2) return dispatch_p<MODE, Real, 2>(f, di, u, du, E, geom, t, s);
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

template <int P, int C, typename State, typename Maker>
int launch_em(const sfx_form_s& f, const DomainIntegral& di, bool diag_only, double* out, int64_t e0, int64_t e1,
              cudaStream_t s) {
  constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
  constexpr int EPW = 32 / NQ;
  if (e1 <= e0) return SFX_OK;
  kernels::DomainArgs<double> a{f.u_lin64.p, nullptr, out, f.conn.p, f.geom64.p, di.state.p, di.params.p,
                                f.nnodes, f.ne, f.t_lin};
  int64_t warps = (e1 - e0 + EPW - 1) / EPW;
  int64_t blocks = (warps * 32 + 127) / 128;
  if (diag_only)
    kernels::element_matrix_kernel<P, C, State, Maker, true><<<unsigned(blocks), 128, 0, s>>>(a, Maker{}, e0, e1);
  else
    kernels::element_matrix_kernel<P, C, State, Maker, false><<<unsigned(blocks), 128, 0, s>>>(a, Maker{}, e0, e1);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("element matrix launch: ") + cudaGetErrorString(err));
  return SFX_OK;
}

template <int P>
int dispatch_em(const sfx_form_s& f, const DomainIntegral& di, bool diag_only, double* out, int64_t e0, int64_t e1,
                cudaStream_t s) {
  switch (di.material) {
    case SFX_MAT_HEAT: return launch_em<P, 1, Nothing, HeatMaker>(f, di, diag_only, out, e0, e1, s);
    case SFX_MAT_NONLINEAR_HEAT: return launch_em<P, 1, Nothing, NonlinearHeatMaker>(f, di, diag_only, out, e0, e1, s);
    case SFX_MAT_THERMAL_TEST: return launch_em<P, 1, Nothing, ThermalTestMaker>(f, di, diag_only, out, e0, e1, s);
    case SFX_MAT_ELASTIC_TEST: return launch_em<P, 3, Nothing, ElasticTestMaker>(f, di, diag_only, out, e0, e1, s);
    case SFX_MAT_NEOHOOKEAN: return launch_em<P, 3, Empty, NeoHookeanMaker>(f, di, diag_only, out, e0, e1, s);
    case SFX_MAT_J2: return launch_em<P, 3, J2::State, J2Maker>(f, di, diag_only, out, e0, e1, s);
  }
  return fail(SFX_ERR_UNSUPPORTED, "unknown material");
}

template <int P>
struct LinearizeFn {
  const sfx_form_s& f;
  DomainIntegral& di;
  double* res_e;
  cudaStream_t s;
  template <int C, typename State, typename Maker>
  int operator()() {
    constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
    constexpr int EPW = 32 / NQ;
    using QF = decltype(Maker{}(nullptr));
    constexpr bool HS = kernels::tangent_has_source<C, State, QF>();
    constexpr bool SYM = sym_of<Maker>::value;
    using Shape = kernels::TangentShape<C, HS, Maker::value_input>;         // FP64: full
    using ShapeP = kernels::TangentShape<C, HS, Maker::value_input, SYM>;  // FP32 / FP16: packed when symmetric
    const size_t n64 = size_t(f.ne) * size_t(Shape::template stride<NQ>);
    const size_t n = size_t(f.ne) * size_t(ShapeP::template stride<NQ>);
    const size_t n16 = size_t(f.ne) * size_t(ShapeP::template stride16<NQ>);
    cudaError_t err = cudaSuccess;
    if (di.D64.n != n64) err = di.D64.alloc(n64);
    if (err == cudaSuccess) {
      if (f.tangent16) {
        di.D32.reset();
        if (di.D16.n != n16) err = di.D16.alloc(n16);
      } else {
        di.D16.reset();
        if (di.D32.n != n) err = di.D32.alloc(n);
      }
    }
    if (err != cudaSuccess) return fail(SFX_ERR_NOMEM, std::string("tangent storage: ") + cudaGetErrorString(err));
    di.tangent_rows = Shape::rows;
    di.tangent_cols = Shape::cols;
    if (f.ne == 0) return SFX_OK;
    kernels::DomainArgs<double> a{f.u_lin64.p, nullptr, nullptr, f.conn.p, f.geom64.p, di.state.p, di.params.p,
                                  f.nnodes, f.ne, f.t_lin};
    int64_t warps = (f.ne + EPW - 1) / EPW;
    int64_t blocks = (warps * 32 + 127) / 128;
    kernels::linearize_kernel<P, C, State, Maker, SYM><<<unsigned(blocks), 128, 0, s>>>(a, Maker{}, di.D64.p, di.D32.p,
                                                                                        di.D16.p, res_e);
    err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("linearize launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

// Bulk-copy staged FP32 action for Q2 (J, or J^T when TRANSPOSE): one
// persistent block per SM with as many warps (up to 24) as fit two-deep rings
// in 220 KB of shared memory, rings up to 4 deep.
template <int C, bool HS, bool VI, bool TRANSPOSE, typename TS, bool SYM>
int launch_tma(const sfx_form_s& f, const float* du, const TS* D, float* E, cudaStream_t s) {
  constexpr int NQ = 27;
  using Shape = kernels::TangentShape<C, HS, VI, SYM>;
  constexpr size_t kSmemBudget = 220 * 1024;
  constexpr size_t stage_bytes = size_t(Shape::template stride_of<NQ, TS>) * sizeof(TS) + 8;
  // 24 warps (the FP16 copy: 768 threads, at most 85 registers each) when
  // two stages of them fit; the FP32 copy gets 16
  constexpr int WARPS = 24 * 2 * stage_bytes <= kSmemBudget   ? 24
                        : 16 * 2 * stage_bytes <= kSmemBudget ? 16
                        : 12 * 2 * stage_bytes <= kSmemBudget ? 12
                        : 8 * 2 * stage_bytes <= kSmemBudget  ? 8
                                                              : 4;
  constexpr int STAGES = int(std::min<size_t>(4, kSmemBudget / (WARPS * stage_bytes)));
  static_assert(STAGES >= 2, "tangent block too large for a two-stage ring");
  constexpr size_t smem = size_t(WARPS) * STAGES * stage_bytes;
  auto kern = kernels::jvp_stored_tma_kernel<C, HS, VI, WARPS, STAGES, TRANSPOSE, TS, SYM>;
  static bool configured = false;  // per instantiation
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("bulk jvp attribute: ") + cudaGetErrorString(e));
    configured = true;
  }
  static int sms = 0;  // SM count, queried once (this launch may sit inside a stream capture)
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const int64_t blocks = std::min<int64_t>((f.ne + WARPS - 1) / WARPS, std::max(sms, 1));
  kern<<<unsigned(blocks), WARPS * 32, smem, s>>>(du, D, f.conn.p, E, f.nnodes, f.ne, f.wait_error.dev);
  return SFX_OK;
}

template <int P, typename Real>
struct StoredJvpFn {
  const sfx_form_s& f;
  const DomainIntegral& di;
  const Real* du;
  const Real* D;
  Real* E;
  cudaStream_t s;
  int64_t e0 = 0, e1 = -1;  // element range [e0, e1) of the FP64 action (default: all)
  template <int C, typename State, typename Maker>
  int operator()() {
    constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
    constexpr int EPW = 32 / NQ;
    using QF = decltype(Maker{}(nullptr));
    constexpr bool HS = kernels::tangent_has_source<C, State, QF>();
    const int64_t first = e0, last = e1 < 0 ? f.ne : e1;
    if (last <= first) return SFX_OK;
    constexpr bool SYM = sym_of<Maker>::value;
    if constexpr (P == 2 && std::is_same<Real, float>::value) {
      if (first != 0 || last != f.ne) return fail(SFX_ERR_UNSUPPORTED, "element ranges are FP64 only");
      const int rc = f.tangent16 ? launch_tma<C, HS, Maker::value_input, false, __half, SYM>(f, du, di.D16.p, E, s)
                                 : launch_tma<C, HS, Maker::value_input, false, float, SYM>(f, du, D, E, s);
      if (rc) return rc;
    } else {
      // the FP64 copy is stored full; the FP32 copy packed when symmetric
      constexpr bool SYMR = SYM && std::is_same<Real, float>::value;
      using Shape = kernels::TangentShape<C, HS, Maker::value_input, SYMR>;
      const int64_t n = last - first;
      int64_t warps = (n + EPW - 1) / EPW;
      int64_t blocks = (warps * 32 + 127) / 128;
      kernels::jvp_stored_kernel<P, C, HS, Maker::value_input, Real, SYMR><<<unsigned(blocks), 128, 0, s>>>(
          du, D + first * Shape::template stride<NQ>, f.conn.p + first * NQ, E + first * C * NQ, f.nnodes, n);
    }
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("stored jvp launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

template <int P, typename Real>
struct StoredJvpTransposeFn {
  const sfx_form_s& f;
  const DomainIntegral& di;
  const Real* v;
  const Real* D;
  Real* E;
  cudaStream_t s;
  template <int C, typename State, typename Maker>
  int operator()() {
    constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
    constexpr int EPW = 32 / NQ;
    using QF = decltype(Maker{}(nullptr));
    constexpr bool HS = kernels::tangent_has_source<C, State, QF>();
    if (f.ne == 0) return SFX_OK;
    constexpr bool SYM = sym_of<Maker>::value;
    if constexpr (P == 2 && std::is_same<Real, float>::value) {
      const int rc = f.tangent16 ? launch_tma<C, HS, Maker::value_input, true, __half, SYM>(f, v, di.D16.p, E, s)
                                 : launch_tma<C, HS, Maker::value_input, true, float, SYM>(f, v, D, E, s);
      if (rc) return rc;
    } else {
      constexpr bool SYMR = SYM && std::is_same<Real, float>::value;
      const int64_t warps = (f.ne + EPW - 1) / EPW;
      const int64_t blocks = (warps * 32 + 127) / 128;
      kernels::jvp_stored_transpose_kernel<P, C, HS, Maker::value_input, Real, SYMR>
          <<<unsigned(blocks), 128, 0, s>>>(v, D, f.conn.p, E, f.nnodes, f.ne);
    }
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("transposed jvp launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

template <int P>
struct DiagFn {
  const sfx_form_s& f;
  const DomainIntegral& di;
  double* E;
  cudaStream_t s;
  template <int C, typename State, typename Maker>
  int operator()() {
    constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
    constexpr int EPW = 32 / NQ;
    using QF = decltype(Maker{}(nullptr));
    constexpr bool HS = kernels::tangent_has_source<C, State, QF>();
    if (f.ne == 0) return SFX_OK;
    int64_t warps = (f.ne + EPW - 1) / EPW;
    int64_t blocks = (warps * 32 + 127) / 128;
    kernels::diag_from_tangent_kernel<P, C, HS, Maker::value_input>
        <<<unsigned(blocks), 128, 0, s>>>(di.D64.p, E, f.ne);  // from the full FP64 copy
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("diagonal launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

}  // namespace

namespace {
template <int P>
struct ShapeJvpFn {
  const sfx_form_s& f;
  const DomainIntegral& di;
  const double* u;
  const double* dshape;
  double* E;
  double t;
  cudaStream_t s;
  template <int C, typename State, typename Maker>
  int operator()() {
    constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
    constexpr int EPW = 32 / NQ;
    if (f.ne == 0) return SFX_OK;
    kernels::DomainArgs<double> a{u, nullptr, E, f.conn.p, nullptr, di.state.p, di.params.p, f.nnodes, f.ne, t};
    const int64_t warps = (f.ne + EPW - 1) / EPW;
    const int64_t blocks = (warps * 32 + 127) / 128;
    kernels::shape_jvp_kernel<P, C, State, Maker><<<unsigned(blocks), 128, 0, s>>>(
        a, Maker{}, f.Xe.p, f.has_shape ? f.shape.p : nullptr, dshape);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("shape jvp launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};
}  // namespace

namespace {
template <int P>
struct ShapeVjpFn {
  const sfx_form_s& f;
  const DomainIntegral& di;
  const double* u;
  const double* lam;
  double* E;
  double t;
  cudaStream_t s;
  template <int C, typename State, typename Maker>
  int operator()() {
    constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
    constexpr int EPW = 32 / NQ;
    if (f.ne == 0) return SFX_OK;
    kernels::DomainArgs<double> a{u, nullptr, nullptr, f.conn.p, nullptr, di.state.p, di.params.p, f.nnodes, f.ne, t};
    const int64_t warps = (f.ne + EPW - 1) / EPW;
    const int64_t blocks = (warps * 32 + 127) / 128;
    kernels::shape_adjoint_kernel<P, C, kernels::SHAPE_VJP, State, Maker><<<unsigned(blocks), 128, 0, s>>>(
        a, Maker{}, f.Xe.p, f.has_shape ? f.shape.p : nullptr, lam, E);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("shape vjp launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};
}  // namespace

int launch_shape_vjp(const sfx_form_s& f, const DomainIntegral& di, const double* u, const double* lam, double* E,
                     double t, cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, ShapeVjpFn<1>{f, di, u, lam, E, t, s});
  if (f.p == 2) return visit_material(di.material, ShapeVjpFn<2>{f, di, u, lam, E, t, s});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_shape_jvp(const sfx_form_s& f, const DomainIntegral& di, const double* u, const double* dshape, double* E,
                     double t, cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, ShapeJvpFn<1>{f, di, u, dshape, E, t, s});
  if (f.p == 2) return visit_material(di.material, ShapeJvpFn<2>{f, di, u, dshape, E, t, s});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_diag_from_tangent(const sfx_form_s& f, const DomainIntegral& di, double* E, cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, DiagFn<1>{f, di, E, s});
  if (f.p == 2) return visit_material(di.material, DiagFn<2>{f, di, E, s});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_linearize(const sfx_form_s& f, DomainIntegral& di, double* res_e, cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, LinearizeFn<1>{f, di, res_e, s});
  if (f.p == 2) return visit_material(di.material, LinearizeFn<2>{f, di, res_e, s});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_jvp_stored(const sfx_form_s& f, const DomainIntegral& di, const double* du, double* E, cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, StoredJvpFn<1, double>{f, di, du, di.D64.p, E, s});
  if (f.p == 2) return visit_material(di.material, StoredJvpFn<2, double>{f, di, du, di.D64.p, E, s});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_jvp_stored_range(const sfx_form_s& f, const DomainIntegral& di, const double* du, double* E, int64_t e0,
                            int64_t e1, cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, StoredJvpFn<1, double>{f, di, du, di.D64.p, E, s, e0, e1});
  if (f.p == 2) return visit_material(di.material, StoredJvpFn<2, double>{f, di, du, di.D64.p, E, s, e0, e1});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_jvp_stored_f32(const sfx_form_s& f, const DomainIntegral& di, const float* du, float* E, cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, StoredJvpFn<1, float>{f, di, du, di.D32.p, E, s});
  if (f.p == 2) return visit_material(di.material, StoredJvpFn<2, float>{f, di, du, di.D32.p, E, s});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_jvp_transpose(const sfx_form_s& f, const DomainIntegral& di, const double* v, double* E, cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, StoredJvpTransposeFn<1, double>{f, di, v, di.D64.p, E, s});
  if (f.p == 2) return visit_material(di.material, StoredJvpTransposeFn<2, double>{f, di, v, di.D64.p, E, s});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_jvp_transpose_f32(const sfx_form_s& f, const DomainIntegral& di, const float* v, float* E,
                             cudaStream_t s) {
  if (f.p == 1) return visit_material(di.material, StoredJvpTransposeFn<1, float>{f, di, v, di.D32.p, E, s});
  if (f.p == 2) return visit_material(di.material, StoredJvpTransposeFn<2, float>{f, di, v, di.D32.p, E, s});
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int launch_element_matrix(const sfx_form_s& f, const DomainIntegral& di, bool diag_only, double* out, int64_t e0,
                          int64_t e1, cudaStream_t s) {
  if (f.p == 1) return dispatch_em<1>(f, di, diag_only, out, e0, e1, s);
  if (f.p == 2) return dispatch_em<2>(f, di, diag_only, out, e0, e1, s);
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int material_info(int material, int* components, int* nparams, int* state_doubles) {
  switch (material) {
    case SFX_MAT_HEAT: *components = 1; *nparams = HeatMaker::nparams; *state_doubles = 0; return SFX_OK;
    case SFX_MAT_NONLINEAR_HEAT: *components = 1; *nparams = NonlinearHeatMaker::nparams; *state_doubles = 0; return SFX_OK;
    case SFX_MAT_THERMAL_TEST: *components = 1; *nparams = 0; *state_doubles = 0; return SFX_OK;
    case SFX_MAT_ELASTIC_TEST: *components = 3; *nparams = 0; *state_doubles = 0; return SFX_OK;
    case SFX_MAT_NEOHOOKEAN: *components = 3; *nparams = NeoHookeanMaker::nparams; *state_doubles = 0; return SFX_OK;
    case SFX_MAT_J2:
      *components = 3;
      *nparams = J2Maker::nparams;
      *state_doubles = int(sizeof(J2::State) / sizeof(double));
      return SFX_OK;
  }
  return fail(SFX_ERR_UNSUPPORTED, "unknown material id");
}

int launch_domain(const sfx_form_s& f, const DomainIntegral& di, int mode, const double* u, const double* du,
                  double* E, double t, cudaStream_t s) {
  switch (mode) {
    case kernels::RESIDUAL: return dispatch<kernels::RESIDUAL, double>(f, di, u, du, E, f.geom64.p, t, s);
    case kernels::RESIDUAL_UPDATE:
      return dispatch<kernels::RESIDUAL_UPDATE, double>(f, di, u, du, E, f.geom64.p, t, s);
    case kernels::JVP: return dispatch<kernels::JVP, double>(f, di, u, du, E, f.geom64.p, t, s);
  }
  return fail(SFX_ERR_INVALID, "bad mode");
}

int launch_domain_jvp_f32(const sfx_form_s& f, const DomainIntegral& di, const float* u, const float* du, float* E,
                          double t, cudaStream_t s) {
  return dispatch<kernels::JVP, float>(f, di, u, du, E, f.geom32.p, t, s);
}

}  // namespace sfx_impl
