// Host-side checks of the product's forward-mode dual numbers and material
// models (include/sfx/dual.hpp, tensor.hpp, materials.hpp: the same headers
// the device kernels compile), in the manner of serac's test_tensor_ad.cpp:
// every directional derivative carried by a dual number is compared with a
// central difference of the value (materials, heat q-functions and the
// boundary models, including the face-Jacobian derivative of the follower
// pressure that the shape-sensitivity kernels use).  Built with g++ by tests/test_ad_host.py;
// prints one line per failed check and exits non-zero on failure.
#include <cmath>
#include <cstdio>
#include <random>
#include <type_traits>

#include "sfx/dual.hpp"
#include "sfx/materials.hpp"
#include "sfx/tensor.hpp"

using namespace sfx;
using S = dual<double, double>;

namespace {

int failures = 0;

void expect_close(const char* what, double ad, double fd, double tol) {
  const double scale = std::fmax(1.0, std::fmax(std::fabs(ad), std::fabs(fd)));
  if (!(std::fabs(ad - fd) <= tol * scale)) {
    std::printf("FAIL %s: dual %.15g, central difference %.15g\n", what, ad, fd);
    failures++;
  }
}

// dual-valued tensor H + eps dH
tensor<S, 3, 3> seeded(const tensor<double, 3, 3>& H, const tensor<double, 3, 3>& dH) {
  tensor<S, 3, 3> out{};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) out[i][j] = S{H[i][j], dH[i][j]};
  return out;
}

tensor<double, 3, 3> shifted(const tensor<double, 3, 3>& H, const tensor<double, 3, 3>& dH, double h) {
  tensor<double, 3, 3> out{};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) out[i][j] = H[i][j] + h * dH[i][j];
  return out;
}

template <typename F>
void check_scalar(const char* what, F f, double x) {
  const double h = 1e-6;
  const auto d = f(S{x, 1.0});
  expect_close(what, d.gradient, (f(x + h) - f(x - h)) / (2 * h), 1e-8);
}

// every entry of a tensor-valued function of H
template <typename F>
void check_tensor_fn(const char* what, F f, const tensor<double, 3, 3>& H, const tensor<double, 3, 3>& dH,
                     double tol = 1e-7) {
  const double h = 1e-6;
  const auto ad = f(seeded(H, dH));
  const auto fp = f(shifted(H, dH, h));
  const auto fm = f(shifted(H, dH, -h));
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) expect_close(what, ad[i][j].gradient, (fp[i][j] - fm[i][j]) / (2 * h), tol);
}

}  // namespace

int main() {
  std::mt19937_64 gen(42);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  auto rand_tensor = [&](double scale) {
    tensor<double, 3, 3> A{};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) A[i][j] = scale * U(gen);
    return A;
  };

  // scalar functions and arithmetic
  check_scalar("sqrt", [](auto x) { using std::sqrt; return sqrt(x); }, 1.7);
  check_scalar("exp", [](auto x) { using std::exp; return exp(x); }, 0.3);
  check_scalar("log", [](auto x) { using std::log; return log(x); }, 2.2);
  check_scalar("log1p", [](auto x) { using std::log1p; return log1p(x); }, -0.2);
  check_scalar("sin", [](auto x) { using std::sin; return sin(x); }, 0.7);
  check_scalar("cos", [](auto x) { using std::cos; return cos(x); }, 0.7);
  check_scalar("pow", [](auto x) { using std::pow; return pow(x, 2.5); }, 1.3);
  check_scalar("quotient", [](auto x) { return (x * x + 1.0) / (2.0 - x); }, 0.4);

  for (int trial = 0; trial < 20; trial++) {
    const auto H = rand_tensor(0.1);
    const auto dH = rand_tensor(1.0);
    // determinant, inverse and det(I + H) - 1 (the cancellation-free form)
    check_tensor_fn("det(I+H)", [](const auto& A) {
      auto d = det(A + Identity<3>());
      tensor<std::decay_t<decltype(d)>, 3, 3> out{};
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[i][j] = d;
      return out;
    }, H, dH);
    check_tensor_fn("inv(I+H)", [](const auto& A) { return inv(A + Identity<3>()); }, H, dH);
    check_tensor_fn("detApIm1", [](const auto& A) {
      auto d = detApIm1(A);
      tensor<std::decay_t<decltype(d)>, 3, 3> out{};
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[i][j] = d;
      return out;
    }, H, dH);
    {  // detApIm1 agrees with det(I + H) - 1
      const double a = detApIm1(H), b = det(H + Identity<3>()) - 1.0;
      expect_close("detApIm1 value", a, b, 1e-14);
    }
    // Neo-Hookean Cauchy stress and its first Piola flux (the functor the kernels call)
    solid_mechanics::NeoHookean nh{1.0, 5.0, 0.25};
    check_tensor_fn("NeoHookean stress", [&](const auto& A) {
      Empty st{};
      return nh(st, A);
    }, H, dH);
    solid_mechanics::MaterialStressFunctor<solid_mechanics::NeoHookean, true> nhf{nh};
    check_tensor_fn("NeoHookean first Piola flux", [&](const auto& A) {
      Empty st{};
      tensor<double, 3> x{};
      using T = std::decay_t<decltype(A[0][0])>;
      return get<1>(nhf(0.0, x, st, tuple{tensor<T, 3>{}, A}));
    }, H, dH);
  }

  // J2 small-strain plasticity: elastic and plastic states, consistent tangent
  using J2 = solid_mechanics::J2SmallStrain<solid_mechanics::LinearHardening>;
  J2 j2{};
  j2.E = 100.0;
  j2.nu = 0.3;
  j2.hardening = solid_mechanics::LinearHardening{1.0, 1.0};
  for (double amplitude : {0.001, 0.05}) {  // elastic, then plastic
    for (int trial = 0; trial < 10; trial++) {
      const auto H = rand_tensor(amplitude);
      const auto dH = rand_tensor(1.0);
      J2::State s0{};
      s0.plastic_strain = rand_tensor(0.002);
      s0.plastic_strain = sym(s0.plastic_strain);
      s0.accumulated_plastic_strain = 0.001;
      check_tensor_fn(amplitude > 0.01 ? "J2 tangent (plastic)" : "J2 tangent (elastic)", [&](const auto& A) {
        J2::State st = s0;
        return j2(st, A);
      }, H, dH, 2e-6);
    }
  }

  // J2 return map (the scalar consistency solve, test_newton.cpp's subject):
  // after a plastic step the stress lies on the yield surface,
  // sqrt(3/2) |dev sigma| = sigma_y + H eqps, to the solver tolerance
  int plastic_draws = 0;
  for (int trial = 0; trial < 20; trial++) {
    const auto H = rand_tensor(0.05);
    J2::State st{};
    const auto sigma = j2(st, H);
    if (st.accumulated_plastic_strain <= 0.0) continue;  // elastic draw
    plastic_draws++;
    const auto s = dev(sigma);
    const double q = std::sqrt(1.5) * norm(s);
    const double yield = j2.hardening.sigma_y + j2.hardening.Hi * st.accumulated_plastic_strain;
    expect_close("J2 consistency", q, yield, 1e-10);
    // the plastic strain increment is deviatoric and along the flow direction
    expect_close("J2 plastic incompressibility", tr(st.plastic_strain), 0.0, 1e-13);
  }
  if (plastic_draws < 10) {
    std::printf("FAIL J2 consistency: only %d plastic draws\n", plastic_draws);
    failures++;
  }

  // heat q-functions: source and flux as functions of (u, grad u)
  for (int trial = 0; trial < 5; trial++) {
    const double u0 = 0.4 * U(gen), du0 = U(gen);
    tensor<double, 3> g0{}, dg0{};
    for (int i = 0; i < 3; i++) {
      g0[i] = U(gen);
      dg0[i] = U(gen);
    }
    heat_transfer::NonlinearHeatIntegrand nl{1.2, 0.7, 0.3};
    auto flux_at = [&](auto uu, auto gg) {
      tensor<double, 3> x{};
      return get<1>(nl(0.0, tuple{x, tensor<double, 3, 3>{}}, tuple{uu, gg}));
    };
    tensor<S, 3> gs{};
    for (int i = 0; i < 3; i++) gs[i] = S{g0[i], dg0[i]};
    const auto ad = flux_at(S{u0, du0}, gs);
    const double h = 1e-6;
    tensor<double, 3> gp{}, gm{};
    for (int i = 0; i < 3; i++) {
      gp[i] = g0[i] + h * dg0[i];
      gm[i] = g0[i] - h * dg0[i];
    }
    const auto fp = flux_at(u0 + h * du0, gp), fm = flux_at(u0 - h * du0, gm);
    for (int i = 0; i < 3; i++) expect_close("nonlinear heat flux", ad[i].gradient, (fp[i] - fm[i]) / (2 * h), 1e-8);
  }

  // boundary models on a face: follower pressure (value of the deformed normal
  // as a function of du/d(s,t), and of the face Jacobian for shape
  // derivatives) and the Robin heat flux
  for (int trial = 0; trial < 5; trial++) {
    tensor<double, 3, 2> J0{}, dU0{}, dir{};
    for (int i = 0; i < 3; i++)
      for (int k = 0; k < 2; k++) {
        J0[i][k] = (i == k ? 1.0 : 0.0) + 0.2 * U(gen);
        dU0[i][k] = 0.05 * U(gen);
        dir[i][k] = U(gen);
      }
    boundary_models::Pressure pr{0.7};
    auto p_of_du = [&](const auto& du) {
      tensor<double, 3> x{};
      using T = std::decay_t<decltype(du[0][0])>;
      return pr(0.0, tuple{x, J0}, tuple{tensor<T, 3>{}, du});
    };
    auto p_of_J = [&](const auto& J) {
      using T = std::decay_t<decltype(J[0][0])>;
      return pr(0.0, tuple{tensor<T, 3>{}, J}, tuple{tensor<double, 3>{}, dU0});
    };
    const double h = 1e-6;
    auto shift = [&](const tensor<double, 3, 2>& A, double hh) {
      tensor<double, 3, 2> out{};
      for (int i = 0; i < 3; i++)
        for (int k = 0; k < 2; k++) out[i][k] = A[i][k] + hh * dir[i][k];
      return out;
    };
    auto seed = [&](const tensor<double, 3, 2>& A) {
      tensor<S, 3, 2> out{};
      for (int i = 0; i < 3; i++)
        for (int k = 0; k < 2; k++) out[i][k] = S{A[i][k], dir[i][k]};
      return out;
    };
    {
      const auto ad = p_of_du(seed(dU0));
      const auto fp = p_of_du(shift(dU0, h)), fm = p_of_du(shift(dU0, -h));
      for (int i = 0; i < 3; i++) expect_close("pressure d/d(du)", ad[i].gradient, (fp[i] - fm[i]) / (2 * h), 1e-8);
    }
    {
      const auto ad = p_of_J(seed(J0));
      const auto fp = p_of_J(shift(J0, h)), fm = p_of_J(shift(J0, -h));
      for (int i = 0; i < 3; i++) expect_close("pressure d/dJ", ad[i].gradient, (fp[i] - fm[i]) / (2 * h), 1e-8);
    }
    boundary_models::HeatFlux hf{0.3, 0.7, 1.1};
    const double u0 = U(gen);
    tensor<double, 3> x{};
    x[0] = 0.4;
    const auto ad = hf(0.0, tuple{x, J0}, tuple{S{u0, 1.0}, tensor<S, 2>{}});
    const auto f1 = hf(0.0, tuple{x, J0}, tuple{u0 + h, tensor<double, 2>{}});
    const auto f2 = hf(0.0, tuple{x, J0}, tuple{u0 - h, tensor<double, 2>{}});
    expect_close("heat flux d/du", ad.gradient, (f1 - f2) / (2 * h), 1e-8);
  }

  if (failures) {
    std::printf("%d checks failed\n", failures);
    return 1;
  }
  std::printf("OK\n");
  return 0;
}
