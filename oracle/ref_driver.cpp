// Checker library built from serac's own header-only element kernels.
//
// This file is test infrastructure: it compiles serac's element-level code
// (domain_integral_kernels.hpp, boundary_integral_kernels.hpp,
// detail/hexahedron_H1.inl, detail/quadrilateral_H1.inl, the tensor / dual AD
// headers and the material models in physics/materials/) against the small
// stand-in headers in oracle/ref_shim/, and exposes a C interface on element
// vectors (E-vectors) so that the CPU restatement in oracle/sfx_oracle.cpp can
// be pinned against the reference arithmetic.  Nothing in the product links it.
//
// Layouts follow the reference:
//   E-vector      : [e][comp][node], node lexicographic (hexahedron_H1.inl:32)
//   positions X_q : [e][3][nq]      (finite_element.hpp:96-99)
//   jacobians J_q : [e][3 (xi)][3 (x)][nq]  (geometric_factors.cpp:52-54)
//   K_e           : [e][trial vdof][test vdof]  (functional.hpp:632-636)
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "serac/numerics/functional/functional.hpp"
#include "serac/numerics/functional/domain_integral_kernels.hpp"
#include "serac/numerics/functional/boundary_integral_kernels.hpp"
#include "serac/physics/materials/solid_material.hpp"
#include "serac/physics/materials/parameterized_solid_material.hpp"
#include "serac/physics/materials/thermal_material.hpp"

using namespace serac;

namespace {

constexpr auto CUBE   = mfem::Geometry::CUBE;
constexpr auto SQUARE = mfem::Geometry::SQUARE;

// ---------------------------------------------------------------- q-functions
// Material ids shared with oracle/sfx_oracle.cpp and the product's C-ABI.
enum Material : int {
  MAT_HEAT            = 0,  // -f source, k grad(u) flux (HeatTransfer + LinearIsotropicConductor + setSource)
  MAT_NEOHOOKEAN      = 1,  // MaterialStressFunctor<NeoHookean>, geometric nonlinearity on
  MAT_J2              = 2,  // MaterialStressFunctor<J2SmallStrain<LinearHardening>>, small strain
  MAT_THERMAL_TEST    = 3,  // linear scalar model with every derivative block populated
  MAT_ELASTIC_TEST    = 4,  // linear vector model with every derivative block populated
  MAT_NONLINEAR_HEAT  = 5,  // k(u) = k0 (1 + beta u^2) conductivity, source -f
};

// heat_transfer.hpp:381-400 (material integrand) plus heat_transfer.hpp:488-505
// (source integrand), merged into one q-function: {-f, -(-k grad u)}.
struct HeatQF {
  double k, f;
  template <typename X, typename T>
  auto operator()(double, X x, T temperature) const
  {
    auto [u, du_dX]       = temperature;
    heat_transfer::LinearIsotropicConductor mat(1.0, 1.0, k);
    auto [hc, heat_flux] = mat(x, u, du_dX);
    (void)hc;
    return serac::tuple{-1.0 * f, -1.0 * heat_flux};
  }
};

struct NonlinearHeatQF {
  double k0, beta, f;
  template <typename X, typename T>
  auto operator()(double, X, T temperature) const
  {
    auto [u, du_dX] = temperature;
    auto kk         = k0 * (1.0 + beta * u * u);
    return serac::tuple{-1.0 * f + 0.0 * u, kk * du_dX};
  }
};

// solid_mechanics.hpp:809-850 with GeometricNonlinearities::On and no
// acceleration field (quasi-static): flux = sigma . F^{-T} det F.
template <typename Material, bool geometric_nonlinearity>
struct StressQF {
  Material material;
  template <typename X, typename State, typename D>
  auto operator()(double, X, State& state, D displacement) const
  {
    auto du_dX  = get<1>(displacement);
    auto stress = material(state, du_dX);
    auto dx_dX  = 0.0 * du_dX + Identity<3>();
    if constexpr (geometric_nonlinearity) {
      dx_dX += du_dX;
    }
    auto flux = dot(stress, transpose(inv(dx_dX))) * det(dx_dX);
    return serac::tuple{zero{}, flux};
  }
};

// Linear scalar / vector models whose tangents populate every derivative
// block (value->source, gradient->source, value->flux, gradient->flux).
struct ThermalTestQF {
  template <typename X, typename T>
  auto operator()(double, X position, T temperature) const
  {
    auto [x, dX_dxi] = position;
    (void)dX_dxi;
    auto [u, du_dx] = temperature;
    tensor<double, 3> d01{0.0, 1.0, 2.0};
    tensor<double, 3> d10{0.0, 2.0, 8.0};
    tensor<double, 3, 3> d11{};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) d11[i][j] = i + j * (j + 1) + 1;
    auto source = 1.0 * u + dot(d01, du_dx) + 0.5 * x[0] * x[1];
    auto flux   = d10 * u + dot(d11, du_dx);
    return serac::tuple{source, flux};
  }
};

struct ElasticTestQF {
  template <typename X, typename T>
  auto operator()(double, X, T displacement) const
  {
    auto [u, du_dx] = displacement;
    tensor<double, 3, 3> d00{};
    tensor<double, 3, 3, 3> d01{}, d10{};
    tensor<double, 3, 3, 3, 3> d11{};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        d00[i][j] = i + 2 * j + 1;
        for (int k = 0; k < 3; k++) {
          d01[i][j][k] = i + 2 * j - k + 1;
          d10[i][j][k] = i + 3 * j - 2 * k;
          for (int l = 0; l < 3; l++) d11[i][j][k][l] = i - j + 2 * k - 3 * l + 1;
        }
      }
    auto source = dot(d00, u) + double_dot(d01, du_dx);
    auto flux   = dot(d10, u) + double_dot(d11, du_dx);
    return serac::tuple{source, flux};
  }
};

// Boundary q-functions (boundary_integral_kernels.hpp:112-156 multiplies the
// returned value by |dX/dxi x dX/deta|).
enum BoundaryMaterial : int {
  BMAT_HEAT_FLUX   = 0,  // scalar: -(q0 + q1 x + alpha u)   (HeatTransfer::setFluxBCs form, Robin term)
  BMAT_TRACTION    = 1,  // vector: -traction(x), traction = t0 + t1 * x[0]  (SolidMechanics::setTraction)
  BMAT_PRESSURE    = 2,  // vector: pressure in the deformed configuration  (SolidMechanics::setPressure)
};

struct HeatFluxBQF {
  double q0, q1, alpha;
  template <typename X, typename T>
  auto operator()(double, X position, T temperature) const
  {
    auto x = get<0>(position);
    auto u = get<0>(temperature);
    return -1.0 * (q0 + q1 * x[0] + alpha * u);
  }
};

struct TractionBQF {
  double t0[3], t1[3];
  template <typename X, typename T>
  auto operator()(double, X position, T displacement) const
  {
    auto x = get<0>(position);
    tensor<double, 3> tr{};
    for (int i = 0; i < 3; i++) tr[i] = t0[i] + t1[i] * x[0];
    return -1.0 * tr + 0.0 * get<0>(displacement);
  }
};

struct PressureBQF {
  double p;
  template <typename X, typename T>
  auto operator()(double, X position, T displacement) const
  {
    auto X0 = get<0>(position);
    auto dX = get<1>(position);
    auto u  = get<0>(displacement);
    auto du = get<1>(displacement);
    // deformed position derivative dx/dxi = dX/dxi + du/dxi
    auto dx = dX + du;
    auto n  = cross(dx);
    (void)X0;
    (void)u;
    return p * (n / norm(cross(dX)));
  }
};

// -------------------------------------------- quantities of interest
// Integrand ids shared with oracle.py (OracleQoI) and the product's C ABI.
enum QoiKind : int {
  QOI_FIELD             = 2,  // w . u
  QOI_NEOHOOKEAN_ENERGY = 3,  // Neo-Hookean stored energy (domain, 3 components)
  QOI_NORMAL_FIELD      = 4,  // u . n (faces, 3 components)
  QOI_POLY_TEST         = 5,  // nonlinear test integrand
};

template <int c, typename U>
auto component_sum(const U& u)
{
  if constexpr (c == 1) {
    return u;
  } else {
    auto s = u[0];
    for (int i = 1; i < c; i++) s = s + u[i];
    return s;
  }
}

template <int c>
struct FieldQoI {
  double w[3];
  template <typename X, typename T>
  auto operator()(double, X, T field) const
  {
    auto u = get<0>(field);
    if constexpr (c == 1) {
      return w[0] * u;
    } else {
      auto s = w[0] * u[0];
      for (int i = 1; i < c; i++) s = s + w[i] * u[i];
      return s;
    }
  }
};

// W = G/2 (|H|^2 + 2 tr H) - G ln J + lambda/2 (ln J)^2 with ln J = log1p(det(I + H) - 1)
struct NeoHookeanEnergyQoI {
  double K, G;
  template <typename X, typename T>
  auto operator()(double, X, T displacement) const
  {
    auto H      = get<1>(displacement);
    using std::log1p;
    auto   lnJ    = log1p(detApIm1(H));
    double lambda = K - (2.0 / 3.0) * G;
    return 0.5 * G * (squared_norm(H) + 2.0 * tr(H)) - G * lnJ + 0.5 * lambda * lnJ * lnJ;
  }
};

// X0^2 + sin X1 + X0 s^3 + (1 + X2)/2 |grad u|^2, s = sum of the components of u
template <int c>
struct PolyQoI {
  template <typename X, typename T>
  auto operator()(double, X position, T field) const
  {
    using std::sin;
    auto x = get<0>(position);
    auto s = component_sum<c>(get<0>(field));
    return x[0] * x[0] + sin(x[1]) + x[0] * s * s * s + 0.5 * (1.0 + x[2]) * squared_norm(get<1>(field));
  }
};

// faces: u . n and X0 - X1 + cos(s X1) + |du/ds|^2 / 4 (du/ds: the first parent direction)
struct NormalFieldQoI {
  template <typename X, typename T>
  auto operator()(double, X position, T displacement) const
  {
    auto n = cross(get<1>(position));
    return dot(get<0>(displacement), n / norm(n));
  }
};

template <int c>
struct PolyFaceQoI {
  template <typename X, typename T>
  auto operator()(double, X position, T field) const
  {
    using std::cos;
    auto x  = get<0>(position);
    auto s  = component_sum<c>(get<0>(field));
    auto du = get<1>(field);
    if constexpr (c == 1) {
      return x[0] - x[1] + cos(s * x[1]) + 0.25 * du[0] * du[0];
    } else {
      auto g = du[0][0] * du[0][0];
      for (int i = 1; i < c; i++) g = g + du[i][0] * du[i][0];
      return x[0] - x[1] + cos(s * x[1]) + 0.25 * g;
    }
  }
};

// per-element values (mode 0) or element gradients dQ_e/du_e (mode 1) of a QoI
template <int p, int c, typename QF>
struct QoiDomainRunner {
  using space   = H1<p, c>;
  using element = finite_element<CUBE, space>;
  using test    = finite_element<CUBE, QOI>;
  static constexpr int Q  = p + 1;
  static constexpr int nq = Q * Q * Q;
  static constexpr int nd = element::ndof * c;
  using deriv_t           = decltype(domain_integral::get_derivative_type<0, 3, space>(QF{}, Nothing{}));

  static void run(int mode, const QF& qf, int ne, double t, const double* uE, const double* X, const double* J,
                  double* out)
  {
    std::vector<deriv_t> derivs(nq);
    axom::Array<Nothing, 2>     arr;
    axom::ArrayView<Nothing, 2> view(arr);
    tuple<element>              trial_elements{};
    int                         elements[1] = {0};
    for (int e = 0; e < ne; e++) {
      std::vector<const double*> inputs{uE + size_t(e) * nd};
      const double*              Xe = X + size_t(e) * 3 * nq;
      const double*              Je = J + size_t(e) * 9 * nq;
      double                     value = 0.0;
      if (mode == 0) {
        domain_integral::evaluation_kernel_impl<NO_DIFFERENTIATION, Q, CUBE>(
            trial_elements, test{}, t, inputs, &value, Xe, Je, qf, view, derivs.data(), elements, 1, false,
            camp::int_seq<int, 0>{});
        out[e] = value;
      } else {
        domain_integral::evaluation_kernel_impl<0, Q, CUBE>(trial_elements, test{}, t, inputs, &value, Xe, Je, qf,
                                                            view, derivs.data(), elements, 1, false,
                                                            camp::int_seq<int, 0>{});
        double* ge = out + size_t(e) * nd;
        std::memset(ge, 0, sizeof(double) * nd);
        ExecArrayView<double, 3, ExecutionSpace::CPU> gview(ge, {1, 1, nd});
        domain_integral::element_gradient_kernel<CUBE, QOI, space, Q>(gview, derivs.data(), elements, 1);
      }
    }
  }
};

template <int p, int c, typename QF>
struct QoiFaceRunner {
  using space   = H1<p, c>;
  using element = finite_element<SQUARE, space>;
  using test    = finite_element<SQUARE, QOI>;
  static constexpr int Q  = p + 1;
  static constexpr int nq = Q * Q;
  static constexpr int nd = element::ndof * c;
  using deriv_t           = decltype(boundary_integral::get_derivative_type<0, 2, space>(QF{}));

  static void run(int mode, const QF& qf, int nf, double t, const double* uF, const double* X, const double* J,
                  double* out)
  {
    std::vector<deriv_t>       derivs(size_t(nf) * nq);
    std::vector<const double*> inputs{uF};
    std::vector<int>           elements(static_cast<size_t>(nf));
    for (int e = 0; e < nf; e++) elements[size_t(e)] = e;
    tuple<element> trial_elements{};
    if (mode == 0) {
      std::memset(out, 0, sizeof(double) * size_t(nf));
      boundary_integral::evaluation_kernel_impl<NO_DIFFERENTIATION, Q, SQUARE>(
          trial_elements, test{}, t, inputs, out, X, J, qf, derivs.data(), elements.data(), uint32_t(nf),
          camp::int_seq<int, 0>{});
      return;
    }
    std::vector<double> values(size_t(nf), 0.0);
    boundary_integral::evaluation_kernel_impl<0, Q, SQUARE>(trial_elements, test{}, t, inputs, values.data(), X, J,
                                                            qf, derivs.data(), elements.data(), uint32_t(nf),
                                                            camp::int_seq<int, 0>{});
    std::memset(out, 0, sizeof(double) * size_t(nf) * nd);
    ExecArrayView<double, 3, ExecutionSpace::CPU> view(out, {nf, 1, nd});
    boundary_integral::element_gradient_kernel<SQUARE, QOI, space, Q>(view, derivs.data(), elements.data(),
                                                                      size_t(nf));
  }
};

template <int p, int c>
int dispatch_qoi(int kind, int boundary, int mode, int n, double t, const double* params, const double* u,
                 const double* X, const double* J, double* out)
{
  if (boundary) {
    if (kind == QOI_FIELD) {
      FieldQoI<c> q{{params[0], c > 1 ? params[1] : 0.0, c > 2 ? params[2] : 0.0}};
      QoiFaceRunner<p, c, FieldQoI<c>>::run(mode, q, n, t, u, X, J, out);
      return 0;
    }
    if (kind == QOI_POLY_TEST) {
      QoiFaceRunner<p, c, PolyFaceQoI<c>>::run(mode, PolyFaceQoI<c>{}, n, t, u, X, J, out);
      return 0;
    }
    if constexpr (c == 3) {
      if (kind == QOI_NORMAL_FIELD) {
        QoiFaceRunner<p, c, NormalFieldQoI>::run(mode, NormalFieldQoI{}, n, t, u, X, J, out);
        return 0;
      }
    }
    return -1;
  }
  if (kind == QOI_FIELD) {
    FieldQoI<c> q{{params[0], c > 1 ? params[1] : 0.0, c > 2 ? params[2] : 0.0}};
    QoiDomainRunner<p, c, FieldQoI<c>>::run(mode, q, n, t, u, X, J, out);
    return 0;
  }
  if (kind == QOI_POLY_TEST) {
    QoiDomainRunner<p, c, PolyQoI<c>>::run(mode, PolyQoI<c>{}, n, t, u, X, J, out);
    return 0;
  }
  if constexpr (c == 3) {
    if (kind == QOI_NEOHOOKEAN_ENERGY) {
      QoiDomainRunner<p, c, NeoHookeanEnergyQoI>::run(mode, NeoHookeanEnergyQoI{params[0], params[1]}, n, t, u, X,
                                                      J, out);
      return 0;
    }
  }
  return -1;
}

// ------------------------------------------------------------ domain kernels
template <int p, int c, typename QF, typename State>
struct DomainRunner {
  using space   = H1<p, c>;
  using element = finite_element<CUBE, space>;
  static constexpr int Q  = p + 1;
  static constexpr int nq = Q * Q * Q;
  static constexpr int nd = element::ndof * c;

  using deriv_t = decltype(domain_integral::get_derivative_type<0, 3, space>(QF{}, State{}));

  static void eval(const QF& qf, double t, const double* uE, const double* X, const double* J, State* state,
                   bool update, double* rE, deriv_t* derivs, bool differentiate)
  {
    std::vector<const double*> inputs{uE};
    int                        elements[1] = {0};
    tuple<element>             trial_elements{};
    if constexpr (std::is_same_v<State, Nothing> || std::is_same_v<State, Empty>) {
      axom::Array<State, 2>     arr;
      axom::ArrayView<State, 2> view(arr);
      if (differentiate) {
        domain_integral::evaluation_kernel_impl<0, Q, CUBE>(trial_elements, element{}, t, inputs, rE, X, J, qf, view,
                                                            derivs, elements, 1, update, camp::int_seq<int, 0>{});
      } else {
        domain_integral::evaluation_kernel_impl<NO_DIFFERENTIATION, Q, CUBE>(
            trial_elements, element{}, t, inputs, rE, X, J, qf, view, derivs, elements, 1, update,
            camp::int_seq<int, 0>{});
      }
    } else {
      axom::ArrayView<State, 2> view(state, {1, nq});
      if (differentiate) {
        domain_integral::evaluation_kernel_impl<0, Q, CUBE>(trial_elements, element{}, t, inputs, rE, X, J, qf, view,
                                                            derivs, elements, 1, update, camp::int_seq<int, 0>{});
      } else {
        domain_integral::evaluation_kernel_impl<NO_DIFFERENTIATION, Q, CUBE>(
            trial_elements, element{}, t, inputs, rE, X, J, qf, view, derivs, elements, 1, update,
            camp::int_seq<int, 0>{});
      }
    }
  }

  // mode 0: residual; 1: residual at u then J(u) du; 2: K_e at u
  static void run(int mode, const QF* qfs, int ne, double t, const double* uE, const double* duE, const double* X,
                  const double* J, State* state, bool update, double* out)
  {
    std::vector<deriv_t> derivs(nq);
    std::vector<double>  scratch(nd);
    for (int e = 0; e < ne; e++) {
      const QF& qf   = qfs[e];
      const double* Xe = X + size_t(e) * 3 * nq;
      const double* Je = J + size_t(e) * 9 * nq;
      State*        se = nullptr;
      if constexpr (!std::is_same_v<State, Nothing>) se = state + size_t(e) * nq;
      if (mode == 0) {
        double* re = out + size_t(e) * nd;
        std::memset(re, 0, sizeof(double) * nd);
        eval(qf, t, uE + size_t(e) * nd, Xe, Je, se, update, re, derivs.data(), false);
      } else {
        // copy the state so that the linearisation does not commit it
        std::vector<State> state_copy(nq);
        State*             sp = se;
        if constexpr (!std::is_same_v<State, Nothing>) {
          for (int q = 0; q < nq; q++) state_copy[size_t(q)] = se[q];
          sp = state_copy.data();
        }
        std::fill(scratch.begin(), scratch.end(), 0.0);
        eval(qf, t, uE + size_t(e) * nd, Xe, Je, sp, false, scratch.data(), derivs.data(), true);
        int elements[1] = {0};
        if (mode == 1) {
          double* re = out + size_t(e) * nd;
          std::memset(re, 0, sizeof(double) * nd);
          domain_integral::action_of_gradient_kernel<Q, CUBE, space, space>(duE + size_t(e) * nd, re, derivs.data(),
                                                                            elements, 1);
        } else {
          double* ke = out + size_t(e) * nd * nd;
          std::memset(ke, 0, sizeof(double) * nd * nd);
          ExecArrayView<double, 3, ExecutionSpace::CPU> view(ke, {1, nd, nd});
          domain_integral::element_gradient_kernel<CUBE, space, space, Q>(view, derivs.data(), elements, 1);
        }
      }
    }
  }
};

template <int p, int c, typename QF>
struct BoundaryRunner {
  using space   = H1<p, c>;
  using element = finite_element<SQUARE, space>;
  static constexpr int Q  = p + 1;
  static constexpr int nq = Q * Q;
  static constexpr int nd = element::ndof * c;
  using deriv_t           = decltype(boundary_integral::get_derivative_type<0, 2, space>(QF{}));

  static void run(int mode, const QF& qf, int nf, double t, const double* uF, const double* duF, const double* X,
                  const double* J, double* out)
  {
    std::vector<deriv_t> derivs(size_t(nf) * nq);
    std::vector<const double*> inputs{uF};
    std::vector<int> elements(static_cast<size_t>(nf));
    for (int e = 0; e < nf; e++) elements[size_t(e)] = e;
    tuple<element> trial_elements{};
    if (mode == 0) {
      std::memset(out, 0, sizeof(double) * size_t(nf) * nd);
      boundary_integral::evaluation_kernel_impl<NO_DIFFERENTIATION, Q, SQUARE>(
          trial_elements, element{}, t, inputs, out, X, J, qf, derivs.data(), elements.data(), uint32_t(nf),
          camp::int_seq<int, 0>{});
      return;
    }
    std::vector<double> scratch(size_t(nf) * nd, 0.0);
    boundary_integral::evaluation_kernel_impl<0, Q, SQUARE>(trial_elements, element{}, t, inputs, scratch.data(), X,
                                                            J, qf, derivs.data(), elements.data(), uint32_t(nf),
                                                            camp::int_seq<int, 0>{});
    if (mode == 1) {
      std::memset(out, 0, sizeof(double) * size_t(nf) * nd);
      boundary_integral::action_of_gradient_kernel<Q, SQUARE, space, space>(duF, out, derivs.data(), elements.data(),
                                                                            size_t(nf));
    } else {
      std::memset(out, 0, sizeof(double) * size_t(nf) * nd * nd);
      ExecArrayView<double, 3, ExecutionSpace::CPU> view(out, {nf, nd, nd});
      boundary_integral::element_gradient_kernel<SQUARE, space, space, Q>(view, derivs.data(), elements.data(),
                                                                          size_t(nf));
    }
  }
};

using J2 = solid_mechanics::J2SmallStrain<solid_mechanics::LinearHardening>;

template <int p>
int dispatch_domain(int mat, int mode, int ne, double t, const double* params, const double* uE, const double* duE,
                    const double* X, const double* J, double* state, int update, double* out)
{
  // params are per element: HEAT {k, f}; NEOHOOKEAN {K, G}; J2 {E, nu, sigma_y, H};
  // NONLINEAR_HEAT {k0, beta, f}; test models take none.
  switch (mat) {
    case MAT_HEAT: {
      std::vector<HeatQF> q(static_cast<size_t>(ne));
      for (int e = 0; e < ne; e++) q[size_t(e)] = HeatQF{params[2 * e], params[2 * e + 1]};
      DomainRunner<p, 1, HeatQF, Nothing>::run(mode, q.data(), ne, t, uE, duE, X, J, nullptr, update, out);
      return 0;
    }
    case MAT_NONLINEAR_HEAT: {
      std::vector<NonlinearHeatQF> q(static_cast<size_t>(ne));
      for (int e = 0; e < ne; e++) q[size_t(e)] = NonlinearHeatQF{params[3 * e], params[3 * e + 1], params[3 * e + 2]};
      DomainRunner<p, 1, NonlinearHeatQF, Nothing>::run(mode, q.data(), ne, t, uE, duE, X, J, nullptr, update, out);
      return 0;
    }
    case MAT_THERMAL_TEST: {
      std::vector<ThermalTestQF> q(static_cast<size_t>(ne));
      DomainRunner<p, 1, ThermalTestQF, Nothing>::run(mode, q.data(), ne, t, uE, duE, X, J, nullptr, update, out);
      return 0;
    }
    case MAT_ELASTIC_TEST: {
      std::vector<ElasticTestQF> q(static_cast<size_t>(ne));
      DomainRunner<p, 3, ElasticTestQF, Nothing>::run(mode, q.data(), ne, t, uE, duE, X, J, nullptr, update, out);
      return 0;
    }
    case MAT_NEOHOOKEAN: {
      using QF = StressQF<solid_mechanics::NeoHookean, true>;
      std::vector<QF> q(static_cast<size_t>(ne));
      for (int e = 0; e < ne; e++) {
        q[size_t(e)].material = solid_mechanics::NeoHookean{1.0, params[2 * e], params[2 * e + 1]};
      }
      std::vector<Empty> st(size_t(ne) * DomainRunner<p, 3, QF, Empty>::nq);
      DomainRunner<p, 3, QF, Empty>::run(mode, q.data(), ne, t, uE, duE, X, J, st.data(), update, out);
      return 0;
    }
    case MAT_J2: {
      using QF = StressQF<J2, false>;
      std::vector<QF> q(static_cast<size_t>(ne));
      for (int e = 0; e < ne; e++) {
        const double* pe      = params + 4 * e;
        q[size_t(e)].material = J2{pe[0], pe[1], solid_mechanics::LinearHardening{pe[2], pe[3]}, 0.0, 1.0};
      }
      // state layout per quadrature point: plastic_strain (9), accumulated_plastic_strain (1)
      static_assert(sizeof(J2::State) == 10 * sizeof(double), "J2 state layout");
      auto* st = reinterpret_cast<J2::State*>(state);
      DomainRunner<p, 3, QF, J2::State>::run(mode, q.data(), ne, t, uE, duE, X, J, st, update, out);
      return 0;
    }
  }
  return -1;
}

template <int p>
int dispatch_boundary(int mat, int mode, int nf, double t, const double* params, const double* uF, const double* duF,
                      const double* X, const double* J, double* out)
{
  switch (mat) {
    case BMAT_HEAT_FLUX: {
      HeatFluxBQF qf{params[0], params[1], params[2]};
      BoundaryRunner<p, 1, HeatFluxBQF>::run(mode, qf, nf, t, uF, duF, X, J, out);
      return 0;
    }
    case BMAT_TRACTION: {
      TractionBQF qf{{params[0], params[1], params[2]}, {params[3], params[4], params[5]}};
      BoundaryRunner<p, 3, TractionBQF>::run(mode, qf, nf, t, uF, duF, X, J, out);
      return 0;
    }
    case BMAT_PRESSURE: {
      PressureBQF qf{params[0]};
      BoundaryRunner<p, 3, PressureBQF>::run(mode, qf, nf, t, uF, duF, X, J, out);
      return 0;
    }
  }
  return -1;
}

template <int Q>
void geometric_factors_q(int ne, const double* Xe, double* Xq, double* Jq)
{
  // geometric_factors.cpp:17-60 with the mesh nodes in H1<1,3> (trilinear)
  using element = finite_element<CUBE, H1<1, 3>>;
  constexpr int nq = Q * Q * Q;
  TensorProductQuadratureRule<Q> rule{};
  auto X = reinterpret_cast<const typename element::dof_type*>(Xe);
  for (int e = 0; e < ne; e++) {
    auto vals = element::interpolate(X[e], rule);
    for (int q = 0; q < nq; q++) {
      auto [value, gradient] = vals[q];
      for (int i = 0; i < 3; i++) {
        Xq[(size_t(e) * 3 + size_t(i)) * nq + size_t(q)] = value[i];
        for (int j = 0; j < 3; j++) Jq[((size_t(e) * 3 + size_t(j)) * 3 + size_t(i)) * nq + size_t(q)] = gradient(i, j);
      }
    }
  }
}

template <int Q>
void face_geometric_factors_q(int nf, const double* Xf, double* Xq, double* Jq)
{
  // geometric_factors.cpp:140-220 for quadrilateral faces with H1<1,3> nodes
  using element = finite_element<SQUARE, H1<1, 3>>;
  constexpr int nq = Q * Q;
  TensorProductQuadratureRule<Q> rule{};
  auto X = reinterpret_cast<const typename element::dof_type*>(Xf);
  for (int e = 0; e < nf; e++) {
    auto vals = element::interpolate(X[e], rule);
    for (int q = 0; q < nq; q++) {
      auto [value, gradient] = vals[q];
      for (int i = 0; i < 3; i++) {
        Xq[(size_t(e) * 3 + size_t(i)) * nq + size_t(q)] = value[i];
        for (int j = 0; j < 2; j++) Jq[((size_t(e) * 2 + size_t(j)) * 3 + size_t(i)) * nq + size_t(q)] = gradient(i, j);
      }
    }
  }
}

}  // namespace

// ------------------------------------------------------ multi-field domain
// SolidMechanics' material integrand with the acceleration and parameter
// fields (solid_mechanics.hpp:809-850 with GeometricNonlinearities::On,
// restated because it is nested in the physics class), evaluated by serac's
// own evaluation_kernel_impl over four trial spaces
// (displacement H1<p,3>, acceleration H1<p,3>, two parameter fields
// H1<p,1>) and differentiated with respect to one of them.
template <typename Material>
struct MultiStressQF {
  Material material;
  template <typename X, typename D, typename A, typename... P>
  auto operator()(double, X, D displacement, A acceleration, P... params) const
  {
    auto  du_dX   = get<1>(displacement);
    auto  d2u_dt2 = get<0>(acceleration);
    Empty state{};
    auto  stress = material(state, du_dX, params...);
    auto  dx_dX  = 0.0 * du_dX + Identity<3>();
    dx_dX += du_dX;
    auto flux = dot(stress, transpose(inv(dx_dX))) * det(dx_dX);
    return serac::tuple{material.density * d2u_dt2, flux};
  }
};

template <int p, uint32_t wrt>
struct MultiRunner {
  using S3 = H1<p, 3>;
  using S1 = H1<p, 1>;
  using E3 = finite_element<CUBE, S3>;
  using E1 = finite_element<CUBE, S1>;
  using QF = MultiStressQF<solid_mechanics::ParameterizedNeoHookeanSolid>;
  static constexpr int Q  = p + 1;
  static constexpr int nq = Q * Q * Q;
  static constexpr int n3 = E3::ndof * 3, n1 = E1::ndof;
  using trial_w           = std::conditional_t<(wrt < 2), S3, S1>;
  static constexpr int nw = wrt < 2 ? n3 : n1;
  using deriv_t           = decltype(domain_integral::get_derivative_type<int(wrt), 3, S3, S3, S1, S1>(QF{}, Nothing{}));

  // mode 0 residual [3 n][e]; 1 Jv wrt; 2 K_e wrt ([e][nw][n3] as the kernel writes it)
  static void run(int mode, int ne, double t, const double* params, const double* uE, const double* aE,
                  const double* kE, const double* gE, const double* dE, const double* X, const double* J, double* out)
  {
    std::vector<deriv_t>        derivs(nq);
    std::vector<double>         scratch(n3);
    axom::Array<Nothing, 2>     arr;
    axom::ArrayView<Nothing, 2> view(arr);
    tuple<E3, E3, E1, E1>       trial_elements{};
    int                         elements[1] = {0};
    for (int e = 0; e < ne; e++) {
      const double* prm = params + size_t(e) * 3;
      QF            qf{solid_mechanics::ParameterizedNeoHookeanSolid{prm[0], prm[1], prm[2]}};
      std::vector<const double*> inputs{uE + size_t(e) * n3, aE + size_t(e) * n3, kE + size_t(e) * n1,
                                        gE + size_t(e) * n1};
      const double* Xe = X + size_t(e) * 3 * nq;
      const double* Je = J + size_t(e) * 9 * nq;
      if (mode == 0) {
        double* re = out + size_t(e) * n3;
        std::memset(re, 0, sizeof(double) * n3);
        domain_integral::evaluation_kernel_impl<NO_DIFFERENTIATION, Q, CUBE>(
            trial_elements, E3{}, t, inputs, re, Xe, Je, qf, view, derivs.data(), elements, 1, false,
            camp::int_seq<int, 0, 1, 2, 3>{});
        continue;
      }
      std::fill(scratch.begin(), scratch.end(), 0.0);
      domain_integral::evaluation_kernel_impl<wrt, Q, CUBE>(trial_elements, E3{}, t, inputs, scratch.data(), Xe, Je,
                                                            qf, view, derivs.data(), elements, 1, false,
                                                            camp::int_seq<int, 0, 1, 2, 3>{});
      if (mode == 1) {
        double* re = out + size_t(e) * n3;
        std::memset(re, 0, sizeof(double) * n3);
        domain_integral::action_of_gradient_kernel<Q, CUBE, S3, trial_w>(dE + size_t(e) * nw, re, derivs.data(),
                                                                         elements, 1);
      } else {
        double* ke = out + size_t(e) * nw * n3;
        std::memset(ke, 0, sizeof(double) * nw * n3);
        ExecArrayView<double, 3, ExecutionSpace::CPU> kview(ke, {1, nw, n3});
        domain_integral::element_gradient_kernel<CUBE, S3, trial_w, Q>(kview, derivs.data(), elements, 1);
      }
    }
  }
};

template <int p>
int dispatch_multi(int mode, int wrt, int ne, double t, const double* params, const double* uE, const double* aE,
                   const double* kE, const double* gE, const double* dE, const double* X, const double* J,
                   double* out)
{
  if (mode == 0) {
    MultiRunner<p, 0>::run(0, ne, t, params, uE, aE, kE, gE, dE, X, J, out);
    return 0;
  }
  switch (wrt) {
    case 0: MultiRunner<p, 0>::run(mode, ne, t, params, uE, aE, kE, gE, dE, X, J, out); return 0;
    case 1: MultiRunner<p, 1>::run(mode, ne, t, params, uE, aE, kE, gE, dE, X, J, out); return 0;
    case 2: MultiRunner<p, 2>::run(mode, ne, t, params, uE, aE, kE, gE, dE, X, J, out); return 0;
    case 3: MultiRunner<p, 3>::run(mode, ne, t, params, uE, aE, kE, gE, dE, X, J, out); return 0;
  }
  return -1;
}

extern "C" {

// Quadrature-point positions and Jacobians of trilinear hexes.
// Xe: [ne][3][8] vertex coordinates in lexicographic order.
int ref_geometric_factors(int Q, int ne, const double* Xe, double* Xq, double* Jq)
{
  if (Q == 2) geometric_factors_q<2>(ne, Xe, Xq, Jq);
  else if (Q == 3) geometric_factors_q<3>(ne, Xe, Xq, Jq);
  else if (Q == 4) geometric_factors_q<4>(ne, Xe, Xq, Jq);
  else return -1;
  return 0;
}

// Same for bilinear quadrilateral faces. Xf: [nf][3][4].
int ref_face_geometric_factors(int Q, int nf, const double* Xf, double* Xq, double* Jq)
{
  if (Q == 2) face_geometric_factors_q<2>(nf, Xf, Xq, Jq);
  else if (Q == 3) face_geometric_factors_q<3>(nf, Xf, Xq, Jq);
  else if (Q == 4) face_geometric_factors_q<4>(nf, Xf, Xq, Jq);
  else return -1;
  return 0;
}

// mode 0: element residuals rE = R_e(u_e); mode 1: element Jacobian action
// dR_e(u_e)[du_e]; mode 2: element stiffness K_e(u_e) [trial][test].
// Q = p + 1 (functional.hpp:193).  J2 state (10 doubles per quadrature point)
// is read, and written back in mode 0 when update != 0.
int ref_domain(int mat, int p, int mode, int ne, double t, const double* params, const double* uE, const double* duE,
               const double* Xq, const double* Jq, double* state, int update, double* out)
{
  try {
    if (p == 1) return dispatch_domain<1>(mat, mode, ne, t, params, uE, duE, Xq, Jq, state, update, out);
    if (p == 2) return dispatch_domain<2>(mat, mode, ne, t, params, uE, duE, Xq, Jq, state, update, out);
    if (p == 3) return dispatch_domain<3>(mat, mode, ne, t, params, uE, duE, Xq, Jq, state, update, out);
  } catch (const std::exception&) {
    return -2;
  }
  return -1;
}

int ref_boundary(int mat, int p, int mode, int nf, double t, const double* params, const double* uF,
                 const double* duF, const double* Xq, const double* Jq, double* out)
{
  try {
    if (p == 1) return dispatch_boundary<1>(mat, mode, nf, t, params, uF, duF, Xq, Jq, out);
    if (p == 2) return dispatch_boundary<2>(mat, mode, nf, t, params, uF, duF, Xq, Jq, out);
  } catch (const std::exception&) {
    return -2;
  }
  return -1;
}

// Quantities of interest (functional_qoi.inl; finite_element<g, QOI>,
// detail/qoi.inl): mode 0 per-element (per-face) values [n], mode 1 element
// gradients dQ_e/du_e [n][c * nodes].  boundary != 0: faces (Xq [n][3][nq],
// Jq [n][2][3][nq]).  Integrands that depend on the field only.
int ref_qoi(int kind, int boundary, int p, int c, int mode, int n, double t, const double* params, const double* u,
            const double* Xq, const double* Jq, double* out)
{
  try {
    if (p == 1 && c == 1) return dispatch_qoi<1, 1>(kind, boundary, mode, n, t, params, u, Xq, Jq, out);
    if (p == 1 && c == 3) return dispatch_qoi<1, 3>(kind, boundary, mode, n, t, params, u, Xq, Jq, out);
    if (p == 2 && c == 1) return dispatch_qoi<2, 1>(kind, boundary, mode, n, t, params, u, Xq, Jq, out);
    if (p == 2 && c == 3) return dispatch_qoi<2, 3>(kind, boundary, mode, n, t, params, u, Xq, Jq, out);
  } catch (const std::exception&) {
    return -2;
  }
  return -1;
}

}  // extern "C"

// The parameterized Neo-Hookean integrand over (u, a, dK, dG) (material 16):
// mode 0 residual -> [e][3 nd]; 1 J_wrt dE -> [e][3 nd]; 2 K_e wrt -> [e][nw][3 nd]
// as element_gradient_kernel writes it.
extern "C" int ref_domain_multi(int mat, int p, int mode, int wrt, int ne, double t, const double* params,
                                const double* uE, const double* aE, const double* kE, const double* gE,
                                const double* dE, const double* Xq, const double* Jq, double* out)
{
  if (mat != 16) return -1;
  try {
    if (p == 1) return dispatch_multi<1>(mode, wrt, ne, t, params, uE, aE, kE, gE, dE, Xq, Jq, out);
    if (p == 2) return dispatch_multi<2>(mode, wrt, ne, t, params, uE, aE, kE, gE, dE, Xq, Jq, out);
  } catch (const std::exception&) {
    return -2;
  }
  return -1;
}
