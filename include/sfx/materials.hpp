// sfx — material q-functions, written once for every number type (double,
// float, dual<...>), evaluated per quadrature point on the device.
//
// They restate serac's material models and physics-module integrands:
//   LinearIsotropicConductor        physics/materials/thermal_material.hpp:20-60
//   HeatIntegrand (material + source) physics/heat_transfer.hpp:381-400, 488-505
//   NeoHookean                      physics/materials/solid_material.hpp:98-127
//   J2SmallStrain<LinearHardening>  physics/materials/solid_material.hpp:132-148, 199-258
//   MaterialStressFunctor           physics/solid_mechanics.hpp:809-850
//   ParameterizedNeoHookean         physics/materials/parameterized_solid_material.hpp:68-110
//   MultiFieldStressFunctor         physics/solid_mechanics.hpp:809-850, 880-893 (acceleration, parameters)
// The q-function call convention is serac's: qf(t, tuple{X, dX_dxi}, [state&,] tuple{value, gradient}).
#pragma once

#include <type_traits>

#include "sfx/dual.hpp"
#include "sfx/tensor.hpp"
#include "sfx/tuple.hpp"

namespace sfx {

/// q-functions without quadrature-point state receive no state argument
struct Nothing {};
/// materials that take a state argument but keep none
struct Empty {};

namespace heat_transfer {

/// thermal_material.hpp:20-60: {rho c_p, -k grad T}
struct LinearIsotropicConductor {
  double density = 1.0, specific_heat_capacity = 1.0, conductivity = 1.0;
  template <typename X, typename T, typename DT>
  SFX_HDI auto operator()(const X&, const T&, const DT& dT_dX) const {
    return tuple{density * specific_heat_capacity, -1.0 * conductivity * dT_dX};
  }
};

/// Steady heat conduction with a uniform source: the sum of HeatTransfer's
/// material integrand {c du/dt, -q} (du/dt = 0) and its source integrand {-f, 0}.
struct HeatIntegrand {
  LinearIsotropicConductor material;
  double source = 0.0;
  template <typename X, typename T>
  SFX_HDI auto operator()(double, const X& x, const T& temperature) const {
    auto u = get<0>(temperature);
    auto du_dX = get<1>(temperature);
    auto q = get<1>(material(x, u, du_dX));
    return tuple{-1.0 * source, -1.0 * q};
  }
};

/// Nonlinear conductivity k(u) = k0 (1 + beta u^2) with a uniform source.
struct NonlinearHeatIntegrand {
  double k0 = 1.0, beta = 0.0, source = 0.0;
  template <typename X, typename T>
  SFX_HDI auto operator()(double, const X&, const T& temperature) const {
    auto u = get<0>(temperature);
    auto du_dX = get<1>(temperature);
    auto k = k0 * (1.0 + beta * u * u);
    return tuple{-1.0 * source, k * du_dX};
  }
};

}  // namespace heat_transfer

namespace solid_mechanics {

/// solid_material.hpp:98-127: Cauchy stress of the compressible Neo-Hookean model
struct NeoHookean {
  using State = Empty;
  double density = 1.0, K = 1.0, G = 1.0;
  template <typename T>
  SFX_HDI auto operator()(State&, const tensor<T, 3, 3>& du_dX) const {
    using std::log1p;
    const auto I = Identity<3>();
    double lambda = K - (2.0 / 3.0) * G;
    auto B_minus_I = dot(du_dX, transpose(du_dX)) + transpose(du_dX) + du_dX;
    auto J_minus_1 = detApIm1(du_dX);
    auto J = J_minus_1 + 1.0;
    return (lambda * log1p(J_minus_1) * I + G * B_minus_I) / J;
  }
};

/// solid_material.hpp:132-148
struct LinearHardening {
  double sigma_y = 1.0, Hi = 0.0;
  template <typename T>
  SFX_HDI auto operator()(const T eqps) const { return sigma_y + Hi * eqps; }
  SFX_HDI double slope(double) const { return Hi; }
};

/// solid_material.hpp:199-258 (J2 small-strain plasticity with isotropic
/// hardening and linear kinematic hardening).  The return map solves the
/// scalar consistency equation by Newton's method in the value part (bounded
/// to 25 iterations and bracketed as in tuple_tensor_dual_functions.hpp:534-650)
/// and propagates derivatives through the implicit function theorem.
template <typename Hardening>
struct J2SmallStrain {
  static constexpr double tol = 1e-10;
  double E = 100.0, nu = 0.3;
  Hardening hardening{};
  double Hk = 0.0, density = 1.0;

  struct State {
    tensor<double, 3, 3> plastic_strain;
    double accumulated_plastic_strain;
  };

  template <typename T>
  SFX_HDI auto operator()(State& state, const tensor<T, 3, 3>& du_dX) const {
    using std::sqrt;
    const auto I = Identity<3>();
    const double K = E / (3.0 * (1.0 - 2.0 * nu));
    const double G = 0.5 * E / (1.0 + nu);
    auto el_strain = sym(du_dX) - state.plastic_strain;
    auto p = K * tr(el_strain);
    auto s = 2.0 * G * dev(el_strain);
    auto sigma_b = (2.0 / 3.0) * Hk * state.plastic_strain;
    auto eta = s - sigma_b;
    auto q = sqrt(1.5) * norm(eta);
    const double eqps_old = state.accumulated_plastic_strain;
    const double qv = double(get_value(q));
    if (qv - hardening(eqps_old) > tol * hardening.sigma_y) {
      // Newton on r(d) = q - (3G + Hk) d - h(eqps_old + d), bracketed in [0, upper]
      double lo = 0.0, hi = (qv - hardening(eqps_old)) / (3.0 * G + Hk);
      double d = 0.0;
      for (int it = 0; it < 25; it++) {
        double r = qv - (3.0 * G + Hk) * d - hardening(eqps_old + d);
        if (r > 0) lo = d; else hi = d;
        if (fabs(r) < tol * hardening.sigma_y) break;
        double drdd = -(3.0 * G + Hk) - hardening.slope(eqps_old + d);
        double dn = d - r / drdd;
        d = (dn > lo && dn < hi) ? dn : 0.5 * (lo + hi);
      }
      double drdd = (3.0 * G + Hk) + hardening.slope(eqps_old + d);
      // delta_eqps as a function of q: d + (q - q.value) / drdd
      auto delta_eqps = (q - qv) * (1.0 / drdd) + d;
      auto Np = 1.5 * eta / q;
      s = s - 2.0 * G * delta_eqps * Np;
      state.accumulated_plastic_strain += double(get_value(delta_eqps));
      state.plastic_strain += double(get_value(delta_eqps)) * get_value_d(Np);
    }
    return s + p * I;
  }

 private:
  template <typename T>
  SFX_HDI static tensor<double, 3, 3> get_value_d(const tensor<T, 3, 3>& A) {
    tensor<double, 3, 3> out{};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) out[i][j] = double(get_value(A[i][j]));
    return out;
  }
};

/// solid_mechanics.hpp:809-850: first Piola flux sigma . F^{-T} det F (with
/// geometric nonlinearity; F = I without it) and inertial source (zero in the
/// quasi-static solve, where acceleration is not a trial field).
template <typename Material, bool geometric_nonlinearity = true>
struct MaterialStressFunctor {
  Material material;
  template <typename X, typename State, typename D>
  SFX_HDI auto operator()(double, const X&, State& state, const D& displacement) const {
    auto du_dX = get<1>(displacement);
    auto stress = material(state, du_dX);
    if constexpr (geometric_nonlinearity) {
      auto dx_dX = du_dX + Identity<3>();
      auto flux = dot(stress, transpose(inv(dx_dX))) * det(dx_dX);
      return tuple{zero{}, flux};
    } else {
      return tuple{zero{}, stress};
    }
  }
};

/// parameterized_solid_material.hpp:68-110 (ParameterizedNeoHookeanSolid):
/// Neo-Hookean Cauchy stress with bulk and shear moduli K0 + dK, G0 + dG,
/// where dK and dG are parameter fields passed as (value, gradient) pairs.
struct ParameterizedNeoHookean {
  using State = Empty;
  double density = 1.0, K0 = 1.0, G0 = 1.0;
  template <typename T, typename PK, typename PG>
  SFX_HDI auto operator()(State&, const tensor<T, 3, 3>& du_dX, const PK& dK, const PG& dG) const {
    using std::log1p;
    const auto I = Identity<3>();
    auto K = K0 + get<0>(dK);
    auto G = G0 + get<0>(dG);
    auto lambda = K - (2.0 / 3.0) * G;
    auto B_minus_I = dot(du_dX, transpose(du_dX)) + transpose(du_dX) + du_dX;
    auto J_minus_1 = detApIm1(du_dX);
    auto J = J_minus_1 + 1.0;
    return (lambda * log1p(J_minus_1) * I + G * B_minus_I) / J;
  }
};

/// solid_mechanics.hpp:809-850 with the acceleration field and parameter
/// fields, as SolidMechanics adds it (DependsOn<0, 1, parameters...>,
/// :880-893): {density * acceleration, sigma . F^{-T} det F}.
template <typename Material, bool geometric_nonlinearity = true>
struct MultiFieldStressFunctor {
  Material material;
  template <typename X, typename State, typename D, typename A, typename... P>
  SFX_HDI auto operator()(double, const X&, State& state, const D& displacement, const A& acceleration,
                          const P&... params) const {
    auto du_dX = get<1>(displacement);
    auto d2u_dt2 = get<0>(acceleration);
    auto stress = material(state, du_dX, params...);
    if constexpr (geometric_nonlinearity) {
      auto dx_dX = du_dX + Identity<3>();
      auto flux = dot(stress, transpose(inv(dx_dX))) * det(dx_dX);
      return tuple{material.density * d2u_dt2, flux};
    } else {
      return tuple{material.density * d2u_dt2, stress};
    }
  }
};

}  // namespace solid_mechanics

namespace test_models {

/// Linear scalar model with every derivative block populated (source and
/// flux depend on both the value and the gradient, plus a position term).
struct ThermalModel {
  template <typename X, typename T>
  SFX_HDI auto operator()(double, const X& position, const T& temperature) const {
    auto x = get<0>(position);
    auto u = get<0>(temperature);
    auto du_dx = get<1>(temperature);
    const tensor<double, 3> d01{{0.0, 1.0, 2.0}};
    const tensor<double, 3> d10{{0.0, 2.0, 8.0}};
    auto d11 = make_tensor<3, 3>([](int i, int j) { return double(i + j * (j + 1) + 1); });
    auto source = 1.0 * u + dot(d01, du_dx) + 0.5 * x[0] * x[1];
    auto flux = u * d10 + dot(d11, du_dx);
    return tuple{source, flux};
  }
};

/// Linear vector model with every derivative block populated.
struct ElasticModel {
  template <typename X, typename T>
  SFX_HDI auto operator()(double, const X&, const T& displacement) const {
    auto u = get<0>(displacement);
    auto du_dx = get<1>(displacement);
    auto d00 = make_tensor<3, 3>([](int i, int j) { return double(i + 2 * j + 1); });
    auto d01 = make_tensor<3, 3, 3>([](int i, int j, int k) { return double(i + 2 * j - k + 1); });
    auto d10 = make_tensor<3, 3, 3>([](int i, int j, int k) { return double(i + 3 * j - 2 * k); });
    auto d11 = make_tensor<3, 3, 3, 3>([](int i, int j, int k, int l) { return double(i - j + 2 * k - 3 * l + 1); });
    auto source = dot(d00, u) + double_dot(d01, du_dx);
    auto flux = dot(d10, u) + double_dot(d11, du_dx);
    return tuple{source, flux};
  }
};

}  // namespace test_models

// --------------------------------------------------------- boundary q-functions
namespace boundary_models {

/// Heat flux with a Robin term: -(q0 + q1 x + alpha u)
struct HeatFlux {
  double q0 = 0.0, q1 = 0.0, alpha = 0.0;
  template <typename X, typename T>
  SFX_HDI auto operator()(double, const X& position, const T& temperature) const {
    auto x = get<0>(position);
    auto u = get<0>(temperature);
    return -1.0 * (alpha * u + (q0 + q1 * x[0]));
  }
};

/// SolidMechanics::setTraction form (solid_mechanics.hpp:1029-1046): -traction(x)
struct Traction {
  double t0[3] = {0, 0, 0}, t1[3] = {0, 0, 0};
  template <typename X, typename T>
  SFX_HDI auto operator()(double, const X& position, const T& displacement) const {
    auto x = get<0>(position);
    auto u = get<0>(displacement);
    using XT = std::decay_t<decltype(x[0])>;  // double, or a dual under a shape derivative
    tensor<XT, 3> tr{};
    for (int i = 0; i < 3; i++) tr[i] = t0[i] + t1[i] * x[0];
    return 0.0 * u - tr;
  }
};

/// SolidMechanics::setPressure form (solid_mechanics.hpp:1063-1099): pressure
/// along the deformed normal, per unit reference area.
struct Pressure {
  double p = 0.0;
  template <typename X, typename T>
  SFX_HDI auto operator()(double, const X& position, const T& displacement) const {
    auto dX = get<1>(position);
    auto du = get<1>(displacement);
    auto n = cross(dX + du);
    return p * (n / norm(cross(dX)));
  }
};

}  // namespace boundary_models

}  // namespace sfx
