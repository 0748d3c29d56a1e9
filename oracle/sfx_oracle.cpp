// ORACLE — test infrastructure only.  CPU restatement of serac::Functional's
// element arithmetic for H1 hexahedra (domain) and quadrilaterals (boundary).
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may
// load this library, and only as the checker / the timed CPU baseline; the
// product never links it.
//
// Parity: pinned against serac's own element kernels compiled from the
// reference sources (oracle/ref_driver.cpp -> oracle/_ref/libserac_ref.so) and
// against the committed fixtures under tests/golden/.
//
// Algorithm (restated, not sum-factorised: every basis function is evaluated
// directly at every quadrature point, an independent route to the same
// numbers as the reference's tensor contractions):
//   - 1-D Gauss-Legendre rule on [0,1] with serac's tabulated digits
//     (numerics/functional/polynomials.hpp:42-52, 271-282)
//   - Lagrange polynomials on Gauss-Lobatto nodes (polynomials.hpp:493-541)
//   - interpolate values and parent gradients (detail/hexahedron_H1.inl:169-228)
//   - parent->physical: grad_x = grad_xi . J^{-1} (finite_element.hpp:246-273)
//   - q-function; derivatives by forward-mode dual numbers seeded on the
//     parent-space inputs, as domain_integral_kernels.hpp:152-220 does
//   - physical->parent: source*detJ, flux . J^{-T} * detJ (finite_element.hpp:287-322)
//   - integrate against the weighted basis (hexahedron_H1.inl:230-280)
//   - Jv by the chain rule on the stored derivative (domain_integral_kernels.hpp:223-304)
//   - K_e column by column, stored [trial vdof][test vdof]
//     (domain_integral_kernels.hpp:327-361, functional.hpp:632-636)
//   - boundary: q-function value times |dX/dxi x dX/deta|
//     (boundary_integral_kernels.hpp:112-156), integrated against the face basis
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------- dual numbers
template <int N>
struct Dual {
  double v;
  double g[N];
};

template <typename S>
struct Traits;
template <>
struct Traits<double> {
  static constexpr int N = 0;
};
template <int N>
struct Traits<Dual<N>> {
  static constexpr int N_ = N;
};

inline double val(double a) { return a; }
template <int N>
inline double val(const Dual<N>& a) { return a.v; }

template <int N>
inline Dual<N> mk(double v) {
  Dual<N> r;
  r.v = v;
  for (int i = 0; i < N; i++) r.g[i] = 0.0;
  return r;
}

template <int N>
inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
  for (int i = 0; i < N; i++) r.g[i] = a.g[i] + b.g[i];
  return r;
}
template <int N>
inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
  for (int i = 0; i < N; i++) r.g[i] = a.g[i] - b.g[i];
  return r;
}
template <int N>
inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
  for (int i = 0; i < N; i++) r.g[i] = -a.g[i];
  return r;
}
template <int N>
inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
  for (int i = 0; i < N; i++) r.g[i] = a.g[i] * b.v + a.v * b.g[i];
  return r;
}
template <int N>
inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  double inv2 = 1.0 / (b.v * b.v);
  for (int i = 0; i < N; i++) r.g[i] = (a.g[i] * b.v - a.v * b.g[i]) * inv2;
  return r;
}
template <int N>
inline Dual<N> operator+(const Dual<N>& a, double b) {
  Dual<N> r = a;
  r.v += b;
  return r;
}
template <int N>
inline Dual<N> operator+(double b, const Dual<N>& a) { return a + b; }
template <int N>
inline Dual<N> operator-(const Dual<N>& a, double b) {
  Dual<N> r = a;
  r.v -= b;
  return r;
}
template <int N>
inline Dual<N> operator-(double b, const Dual<N>& a) { return -a + b; }
template <int N>
inline Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
  for (int i = 0; i < N; i++) r.g[i] = a.g[i] * b;
  return r;
}
template <int N>
inline Dual<N> operator*(double b, const Dual<N>& a) { return a * b; }
template <int N>
inline Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v / b;
  for (int i = 0; i < N; i++) r.g[i] = a.g[i] / b;
  return r;
}
template <int N>
inline Dual<N> log1p(const Dual<N>& a) {
  Dual<N> r;
  r.v = std::log1p(a.v);
  double d = 1.0 / (1.0 + a.v);
  for (int i = 0; i < N; i++) r.g[i] = a.g[i] * d;
  return r;
}
template <int N>
inline Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = std::sqrt(a.v);
  double d = 0.5 / r.v;
  for (int i = 0; i < N; i++) r.g[i] = a.g[i] * d;
  return r;
}
using std::log1p;
using std::sqrt;

// a zero of type S
template <typename S>
inline S Z() { return S{}; }
template <>
inline double Z<double>() { return 0.0; }

template <typename S>
inline S C(double v) { return S{} + v; }
template <>
inline double C<double>(double v) { return v; }

// ------------------------------------------------------- small dense algebra
template <typename S>
struct M3 {
  S a[3][3];
};

template <typename S>
inline S det3(const M3<S>& m) {
  return m.a[0][0] * m.a[1][1] * m.a[2][2] + m.a[0][1] * m.a[1][2] * m.a[2][0] + m.a[0][2] * m.a[1][0] * m.a[2][1] -
         m.a[0][0] * m.a[1][2] * m.a[2][1] - m.a[0][1] * m.a[1][0] * m.a[2][2] - m.a[0][2] * m.a[1][1] * m.a[2][0];
}

template <typename S>
inline M3<S> inv3(const M3<S>& m) {
  S d = det3(m);
  M3<S> r;
  r.a[0][0] = (m.a[1][1] * m.a[2][2] - m.a[1][2] * m.a[2][1]) / d;
  r.a[0][1] = (m.a[0][2] * m.a[2][1] - m.a[0][1] * m.a[2][2]) / d;
  r.a[0][2] = (m.a[0][1] * m.a[1][2] - m.a[0][2] * m.a[1][1]) / d;
  r.a[1][0] = (m.a[1][2] * m.a[2][0] - m.a[1][0] * m.a[2][2]) / d;
  r.a[1][1] = (m.a[0][0] * m.a[2][2] - m.a[0][2] * m.a[2][0]) / d;
  r.a[1][2] = (m.a[0][2] * m.a[1][0] - m.a[0][0] * m.a[1][2]) / d;
  r.a[2][0] = (m.a[1][0] * m.a[2][1] - m.a[1][1] * m.a[2][0]) / d;
  r.a[2][1] = (m.a[0][1] * m.a[2][0] - m.a[0][0] * m.a[2][1]) / d;
  r.a[2][2] = (m.a[0][0] * m.a[1][1] - m.a[0][1] * m.a[1][0]) / d;
  return r;
}

// det(I + A) - 1 without cancellation (tensor.hpp:1266-1290 states the identity
// det(I+A)-1 = tr A + (tr(A)^2 - tr(A^2))/2 + det A)
template <typename S>
inline S det_ap_im1(const M3<S>& A) {
  S trA = A.a[0][0] + A.a[1][1] + A.a[2][2];
  S trA2 = Z<S>();
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) trA2 = trA2 + A.a[i][j] * A.a[j][i];
  return trA + 0.5 * (trA * trA - trA2) + det3(A);
}

// ------------------------------------------------------------- quadrature
// serac's tabulated 1-D Gauss-Legendre rule on [0, 1].
const double* gl_points(int q) {
  static const double p1[] = {0.5};
  static const double p2[] = {0.2113248654051871, 0.7886751345948129};
  static const double p3[] = {0.1127016653792583, 0.500000000000000, 0.887298334620742};
  static const double p4[] = {0.0694318442029737, 0.330009478207572, 0.669990521792428, 0.930568155797026};
  switch (q) {
    case 1: return p1;
    case 2: return p2;
    case 3: return p3;
    case 4: return p4;
  }
  return nullptr;
}
const double* gl_weights(int q) {
  static const double w1[] = {1.0};
  static const double w2[] = {0.5, 0.5};
  static const double w3[] = {0.277777777777778, 0.444444444444444, 0.277777777777778};
  static const double w4[] = {0.173927422568727, 0.326072577431273, 0.326072577431273, 0.173927422568727};
  switch (q) {
    case 1: return w1;
    case 2: return w2;
    case 3: return w3;
    case 4: return w4;
  }
  return nullptr;
}

// Lagrange basis on the Gauss-Lobatto nodes of [0,1] (n = p+1 nodes), and its
// derivative, by the product formula.
void gll_nodes(int n, double* x) {
  if (n == 2) {
    x[0] = 0.0;
    x[1] = 1.0;
  } else if (n == 3) {
    x[0] = 0.0;
    x[1] = 0.5;
    x[2] = 1.0;
  } else {
    x[0] = 0.0;
    x[1] = 0.5 - 0.5 / std::sqrt(5.0);
    x[2] = 0.5 + 0.5 / std::sqrt(5.0);
    x[3] = 1.0;
  }
}
void lagrange(int n, double t, double* phi, double* dphi) {
  double x[4];
  gll_nodes(n, x);
  for (int i = 0; i < n; i++) {
    double v = 1.0, d = 0.0;
    for (int j = 0; j < n; j++) {
      if (j == i) continue;
      double term = (t - x[j]) / (x[i] - x[j]);
      double dterm = 1.0 / (x[i] - x[j]);
      d = d * term + v * dterm;
      v = v * term;
    }
    phi[i] = v;
    dphi[i] = d;
  }
}

// ---------------------------------------------------------------- materials
enum Material : int {
  MAT_HEAT = 0,
  MAT_NEOHOOKEAN = 1,
  MAT_J2 = 2,
  MAT_THERMAL_TEST = 3,
  MAT_ELASTIC_TEST = 4,
  MAT_NONLINEAR_HEAT = 5,
};

// q-function inputs/outputs for up to 3 components, scalar type S
template <typename S>
struct QIn {
  double x[3];
  double J[3][3];
  S u[3];
  S du[3][3];  // physical gradient du[c][j] = d u_c / d x_j
};
template <typename S>
struct QOut {
  S s[3];
  S f[3][3];
  bool has_source;
};

struct J2State {
  double ep[3][3];
  double eqps;
};

// heat_transfer.hpp:381-400 + 488-505 + thermal_material.hpp:20-60
template <typename S>
void qf_heat(const double* prm, const QIn<S>& in, QOut<S>& out) {
  double k = prm[0], f = prm[1];
  out.has_source = true;
  out.s[0] = C<S>(-f);
  for (int j = 0; j < 3; j++) out.f[0][j] = k * in.du[0][j];
}

template <typename S>
void qf_nonlinear_heat(const double* prm, const QIn<S>& in, QOut<S>& out) {
  double k0 = prm[0], beta = prm[1], f = prm[2];
  out.has_source = true;
  out.s[0] = C<S>(-f) + 0.0 * in.u[0];
  S kk = k0 * (1.0 + beta * in.u[0] * in.u[0]);
  for (int j = 0; j < 3; j++) out.f[0][j] = kk * in.du[0][j];
}

template <typename S>
void qf_thermal_test(const double*, const QIn<S>& in, QOut<S>& out) {
  const double d01[3] = {0.0, 1.0, 2.0};
  const double d10[3] = {0.0, 2.0, 8.0};
  out.has_source = true;
  S s = 1.0 * in.u[0];
  for (int j = 0; j < 3; j++) s = s + d01[j] * in.du[0][j];
  out.s[0] = s + 0.5 * in.x[0] * in.x[1];
  for (int i = 0; i < 3; i++) {
    S f = d10[i] * in.u[0];
    for (int j = 0; j < 3; j++) f = f + double(i + j * (j + 1) + 1) * in.du[0][j];
    out.f[0][i] = f;
  }
}

template <typename S>
void qf_elastic_test(const double*, const QIn<S>& in, QOut<S>& out) {
  out.has_source = true;
  for (int i = 0; i < 3; i++) {
    S s = Z<S>();
    for (int j = 0; j < 3; j++) {
      s = s + double(i + 2 * j + 1) * in.u[j];
      for (int k = 0; k < 3; k++) s = s + double(i + 2 * j - k + 1) * in.du[j][k];
    }
    out.s[i] = s;
    for (int j = 0; j < 3; j++) {
      S f = Z<S>();
      for (int k = 0; k < 3; k++) {
        f = f + double(i + 3 * j - 2 * k) * in.u[k];
        for (int l = 0; l < 3; l++) f = f + double(i - j + 2 * k - 3 * l + 1) * in.du[k][l];
      }
      out.f[i][j] = f;
    }
  }
}

// solid_material.hpp:98-127 (NeoHookean) inside solid_mechanics.hpp:809-850
// (MaterialStressFunctor, geometric nonlinearity on)
template <typename S>
void qf_neohookean(const double* prm, const QIn<S>& in, QOut<S>& out) {
  double K = prm[0], G = prm[1];
  out.has_source = false;
  M3<S> H;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) H.a[i][j] = in.du[i][j];
  double lambda = K - (2.0 / 3.0) * G;
  M3<S> BmI;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      S hh = Z<S>();
      for (int k = 0; k < 3; k++) hh = hh + H.a[i][k] * H.a[j][k];
      BmI.a[i][j] = hh + H.a[j][i] + H.a[i][j];
    }
  S Jm1 = det_ap_im1(H);
  S Jd = Jm1 + 1.0;
  S lg = log1p(Jm1);
  M3<S> sigma;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) sigma.a[i][j] = (lambda * lg * (i == j ? 1.0 : 0.0) + G * BmI.a[i][j]) / Jd;
  M3<S> F = H;
  for (int i = 0; i < 3; i++) F.a[i][i] = F.a[i][i] + 1.0;
  M3<S> Fi = inv3(F);
  S dF = det3(F);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      S acc = Z<S>();
      for (int k = 0; k < 3; k++) acc = acc + sigma.a[i][k] * Fi.a[j][k];
      out.f[i][j] = acc * dF;
    }
}

// solid_material.hpp:199-258 (J2SmallStrain<LinearHardening>, Hk = 0) with
// geometric nonlinearity off: flux = Cauchy stress.  The return map's scalar
// equation is linear in the plastic increment for linear hardening, so the
// Newton solve of tuple_tensor_dual_functions.hpp:534-650 ends after one
// step; its derivative follows from the implicit function theorem.
template <typename S>
void qf_j2(const double* prm, J2State& st, bool update, const QIn<S>& in, QOut<S>& out) {
  double E = prm[0], nu = prm[1], sy = prm[2], Hi = prm[3];
  const double tol = 1e-10;
  double K = E / (3.0 * (1.0 - 2.0 * nu));
  double G = 0.5 * E / (1.0 + nu);
  out.has_source = false;
  M3<S> el;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) el.a[i][j] = 0.5 * (in.du[i][j] + in.du[j][i]) - st.ep[i][j];
  S tr = el.a[0][0] + el.a[1][1] + el.a[2][2];
  S p = K * tr;
  M3<S> s;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) s.a[i][j] = 2.0 * G * (el.a[i][j] - (i == j ? (tr / 3.0) : Z<S>()));
  // eta = s (no kinematic hardening)
  S nrm2 = Z<S>();
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) nrm2 = nrm2 + s.a[i][j] * s.a[i][j];
  S q = std::sqrt(1.5) * sqrt(nrm2);
  double eqps_old = st.eqps;
  double r0 = val(q) - (sy + Hi * eqps_old);
  if (r0 > tol * sy) {
    S dq = (q - (sy + Hi * eqps_old)) / (3.0 * G + Hi);
    M3<S> Np;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Np.a[i][j] = 1.5 * s.a[i][j] / q;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) s.a[i][j] = s.a[i][j] - 2.0 * G * dq * Np.a[i][j];
    if (update) {
      st.eqps += val(dq);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) st.ep[i][j] += val(dq) * val(Np.a[i][j]);
    }
  }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) out.f[i][j] = s.a[i][j] + (i == j ? p : Z<S>());
}

template <typename S>
void call_qf(int mat, const double* prm, J2State* st, bool update, const QIn<S>& in, QOut<S>& out) {
  switch (mat) {
    case MAT_HEAT: qf_heat(prm, in, out); break;
    case MAT_NONLINEAR_HEAT: qf_nonlinear_heat(prm, in, out); break;
    case MAT_THERMAL_TEST: qf_thermal_test(prm, in, out); break;
    case MAT_ELASTIC_TEST: qf_elastic_test(prm, in, out); break;
    case MAT_NEOHOOKEAN: qf_neohookean(prm, in, out); break;
    case MAT_J2: qf_j2(prm, *st, update, in, out); break;
  }
}

int components_of(int mat) {
  return (mat == MAT_HEAT || mat == MAT_NONLINEAR_HEAT || mat == MAT_THERMAL_TEST) ? 1 : 3;
}
int params_of(int mat) {
  switch (mat) {
    case MAT_HEAT: return 2;
    case MAT_NEOHOOKEAN: return 2;
    case MAT_J2: return 4;
    case MAT_NONLINEAR_HEAT: return 3;
  }
  return 0;
}

// ------------------------------------------------------------ domain kernel
struct Basis3 {
  int n, q, nd, nq;
  std::vector<double> phi;   // [qp][node]
  std::vector<double> dphi;  // [qp][node][3]
  std::vector<double> w;     // [qp]
  Basis3(int p) : n(p + 1), q(p + 1) {
    nd = n * n * n;
    nq = q * q * q;
    phi.resize(size_t(nq * nd));
    dphi.resize(size_t(nq * nd * 3));
    w.resize(size_t(nq));
    const double* pts = gl_points(q);
    const double* wts = gl_weights(q);
    double B[4][4], G[4][4];
    for (int i = 0; i < q; i++) lagrange(n, pts[i], B[i], G[i]);
    for (int qz = 0; qz < q; qz++)
      for (int qy = 0; qy < q; qy++)
        for (int qx = 0; qx < q; qx++) {
          int Q = (qz * q + qy) * q + qx;
          w[size_t(Q)] = wts[qx] * wts[qy] * wts[qz];
          for (int kz = 0; kz < n; kz++)
            for (int ky = 0; ky < n; ky++)
              for (int kx = 0; kx < n; kx++) {
                int a = (kz * n + ky) * n + kx;
                size_t o = size_t(Q * nd + a);
                phi[o] = B[qx][kx] * B[qy][ky] * B[qz][kz];
                dphi[o * 3 + 0] = G[qx][kx] * B[qy][ky] * B[qz][kz];
                dphi[o * 3 + 1] = B[qx][kx] * G[qy][ky] * B[qz][kz];
                dphi[o * 3 + 2] = B[qx][kx] * B[qy][ky] * G[qz][kz];
              }
        }
  }
};

// Evaluate the q-function at one quadrature point with dual seeds on the
// parent-space inputs; returns D (the derivative of the parent-space
// source/flux w.r.t. the parent-space value/gradient) and the value.
// Layout of the 4c inputs / 4c outputs: [value c][gradient c x 3].
template <int c>
void qp_linearise(int mat, const double* prm, J2State* st, const double* xq, const double J[3][3], const double* uval,
                  const double (*ugrad)[3], double* out_val, double* D) {
  constexpr int N = 4 * c;
  using S = Dual<N>;
  M3<double> Jm;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Jm.a[i][j] = J[i][j];
  M3<double> Ji = inv3(Jm);
  double dv = det3(Jm);
  QIn<S> in;
  for (int i = 0; i < 3; i++) {
    in.x[i] = xq[i];
    for (int j = 0; j < 3; j++) in.J[i][j] = J[i][j];
  }
  S g[3][3];
  for (int i = 0; i < c; i++) {
    in.u[i] = mk<N>(uval[i]);
    in.u[i].g[i] = 1.0;
    for (int j = 0; j < 3; j++) {
      g[i][j] = mk<N>(ugrad[i][j]);
      g[i][j].g[c + 3 * i + j] = 1.0;
    }
  }
  for (int i = 0; i < c; i++)
    for (int j = 0; j < 3; j++) {
      S acc = mk<N>(0.0);
      for (int k = 0; k < 3; k++) acc = acc + g[i][k] * Ji.a[k][j];
      in.du[i][j] = acc;
    }
  QOut<S> out;
  out.has_source = false;
  for (int i = 0; i < 3; i++) {
    out.s[i] = mk<N>(0.0);
    for (int j = 0; j < 3; j++) out.f[i][j] = mk<N>(0.0);
  }
  J2State local;
  if (st) local = *st;
  call_qf<S>(mat, prm, st ? &local : nullptr, false, in, out);
  // physical -> parent
  for (int i = 0; i < c; i++) {
    S s = out.has_source ? out.s[i] * dv : mk<N>(0.0);
    out_val[i] = s.v;
    for (int n = 0; n < N; n++) D[i * N + n] = s.g[n];
    for (int k = 0; k < 3; k++) {
      S acc = mk<N>(0.0);
      for (int m = 0; m < 3; m++) acc = acc + out.f[i][m] * Ji.a[k][m];
      acc = acc * dv;
      out_val[c + 3 * i + k] = acc.v;
      for (int n = 0; n < N; n++) D[(c + 3 * i + k) * N + n] = acc.g[n];
    }
  }
}

template <int c>
void domain_element(int mat, int p, int mode, double t, const double* prm, const Basis3& b, const double* ue,
                    const double* due, const double* Xq, const double* Jq, J2State* st, bool update, double* out) {
  (void)t;
  const int nd = b.nd, nq = b.nq;
  constexpr int N = 4 * c;
  std::vector<double> Dq;
  if (mode == 2) Dq.assign(size_t(nq) * N * N, 0.0);
  if (mode == 0) std::memset(out, 0, sizeof(double) * size_t(nd * c));
  if (mode == 1) std::memset(out, 0, sizeof(double) * size_t(nd * c));
  (void)p;
  for (int q = 0; q < nq; q++) {
    const double* phi = &b.phi[size_t(q * nd)];
    const double* dphi = &b.dphi[size_t(q * nd * 3)];
    double uval[3] = {0, 0, 0}, ugrad[3][3] = {};
    for (int i = 0; i < c; i++)
      for (int a = 0; a < nd; a++) {
        double ua = ue[i * nd + a];
        uval[i] += ua * phi[a];
        for (int j = 0; j < 3; j++) ugrad[i][j] += ua * dphi[a * 3 + j];
      }
    double J[3][3], xq[3];
    for (int i = 0; i < 3; i++) {
      xq[i] = Xq[i * nq + q];
      for (int j = 0; j < 3; j++) J[i][j] = Jq[(j * 3 + i) * nq + q];  // J[i][j] = dx_i/dxi_j
    }
    double w = b.w[size_t(q)];
    J2State* sq = st ? st + q : nullptr;
    if (mode == 0) {
      // value only, plain doubles
      M3<double> Jm;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Jm.a[i][j] = J[i][j];
      M3<double> Ji = inv3(Jm);
      double dv = det3(Jm);
      QIn<double> in;
      for (int i = 0; i < 3; i++) {
        in.x[i] = xq[i];
        for (int j = 0; j < 3; j++) in.J[i][j] = J[i][j];
      }
      for (int i = 0; i < c; i++) {
        in.u[i] = uval[i];
        for (int j = 0; j < 3; j++) {
          double acc = 0.0;
          for (int k = 0; k < 3; k++) acc += ugrad[i][k] * Ji.a[k][j];
          in.du[i][j] = acc;
        }
      }
      QOut<double> o{};
      call_qf<double>(mat, prm, sq, update, in, o);
      for (int i = 0; i < c; i++) {
        double s = o.has_source ? o.s[i] * dv : 0.0;
        double fp[3];
        for (int k = 0; k < 3; k++) {
          double acc = 0.0;
          for (int m = 0; m < 3; m++) acc += o.f[i][m] * Ji.a[k][m];
          fp[k] = acc * dv;
        }
        for (int a = 0; a < nd; a++)
          out[i * nd + a] += w * (s * phi[a] + fp[0] * dphi[a * 3] + fp[1] * dphi[a * 3 + 1] + fp[2] * dphi[a * 3 + 2]);
      }
      continue;
    }
    double vals[4 * c];
    double D[N * N];
    qp_linearise<c>(mat, prm, sq, xq, J, uval, ugrad, vals, D);
    if (mode == 1) {
      double din[N];
      for (int i = 0; i < N; i++) din[i] = 0.0;
      for (int i = 0; i < c; i++)
        for (int a = 0; a < nd; a++) {
          double da = due[i * nd + a];
          din[i] += da * phi[a];
          for (int j = 0; j < 3; j++) din[c + 3 * i + j] += da * dphi[a * 3 + j];
        }
      double dout[N];
      for (int r = 0; r < N; r++) {
        double acc = 0.0;
        for (int s = 0; s < N; s++) acc += D[r * N + s] * din[s];
        dout[r] = acc;
      }
      for (int i = 0; i < c; i++)
        for (int a = 0; a < nd; a++)
          out[i * nd + a] += w * (dout[i] * phi[a] + dout[c + 3 * i] * dphi[a * 3] + dout[c + 3 * i + 1] * dphi[a * 3 + 1] +
                                  dout[c + 3 * i + 2] * dphi[a * 3 + 2]);
    } else {
      std::memcpy(&Dq[size_t(q) * N * N], D, sizeof(D));
    }
  }
  if (mode == 2) {
    // K[trial (jc, b)][test (ic, a)]
    const int ndof = nd * c;
    std::memset(out, 0, sizeof(double) * size_t(ndof) * size_t(ndof));
    for (int q = 0; q < nq; q++) {
      const double* phi = &b.phi[size_t(q * nd)];
      const double* dphi = &b.dphi[size_t(q * nd * 3)];
      const double* D = &Dq[size_t(q) * N * N];
      double w = b.w[size_t(q)];
      for (int jc = 0; jc < c; jc++)
        for (int bb = 0; bb < nd; bb++) {
          double din[N];
          for (int i = 0; i < N; i++) din[i] = 0.0;
          din[jc] = phi[bb];
          for (int j = 0; j < 3; j++) din[c + 3 * jc + j] = dphi[bb * 3 + j];
          double dout[N];
          for (int r = 0; r < N; r++) {
            double acc = 0.0;
            for (int s = 0; s < N; s++) acc += D[r * N + s] * din[s];
            dout[r] = acc;
          }
          double* col = out + size_t(jc * nd + bb) * size_t(ndof);
          for (int ic = 0; ic < c; ic++)
            for (int a = 0; a < nd; a++)
              col[ic * nd + a] += w * (dout[ic] * phi[a] + dout[c + 3 * ic] * dphi[a * 3] +
                                       dout[c + 3 * ic + 1] * dphi[a * 3 + 1] + dout[c + 3 * ic + 2] * dphi[a * 3 + 2]);
        }
    }
  }
}

// ---------------------------------------------------------- boundary kernel
enum BoundaryMaterial : int { BMAT_HEAT_FLUX = 0, BMAT_TRACTION = 1, BMAT_PRESSURE = 2 };

template <typename S>
void bqf(int mat, const double* prm, const double* x, const double J[3][2], const S* u, const S (*du)[2], S* out) {
  if (mat == BMAT_HEAT_FLUX) {
    out[0] = -1.0 * (C<S>(prm[0] + prm[1] * x[0]) + prm[2] * u[0]);
  } else if (mat == BMAT_TRACTION) {
    for (int i = 0; i < 3; i++) out[i] = C<S>(-(prm[i] + prm[3 + i] * x[0])) + 0.0 * u[i];
  } else {
    // pressure p * n(deformed) / |n(reference)|
    S dx[3][2];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 2; j++) dx[i][j] = C<S>(J[i][j]) + du[i][j];
    S n[3];
    n[0] = dx[1][0] * dx[2][1] - dx[2][0] * dx[1][1];
    n[1] = dx[2][0] * dx[0][1] - dx[0][0] * dx[2][1];
    n[2] = dx[0][0] * dx[1][1] - dx[1][0] * dx[0][1];
    double n0[3] = {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1],
                    J[0][0] * J[1][1] - J[1][0] * J[0][1]};
    double nn = std::sqrt(n0[0] * n0[0] + n0[1] * n0[1] + n0[2] * n0[2]);
    for (int i = 0; i < 3; i++) out[i] = prm[0] * (n[i] / nn);
  }
}

template <int c>
void boundary_face(int mat, int p, int mode, const double* prm, const double* ue, const double* due, const double* Xq,
                   const double* Jq, double* out) {
  const int n = p + 1, q = p + 1, nd = n * n, nq = q * q;
  const double* pts = gl_points(q);
  const double* wts = gl_weights(q);
  double B[4][4], G[4][4];
  for (int i = 0; i < q; i++) lagrange(n, pts[i], B[i], G[i]);
  constexpr int N = 3 * c;
  const int ndof = nd * c;
  if (mode == 2) std::memset(out, 0, sizeof(double) * size_t(ndof * ndof));
  else std::memset(out, 0, sizeof(double) * size_t(ndof));
  for (int qy = 0; qy < q; qy++)
    for (int qx = 0; qx < q; qx++) {
      int Q = qy * q + qx;
      double w = wts[qx] * wts[qy];
      double phi[16], dphi[16][2];
      for (int ky = 0; ky < n; ky++)
        for (int kx = 0; kx < n; kx++) {
          int a = ky * n + kx;
          phi[a] = B[qx][kx] * B[qy][ky];
          dphi[a][0] = G[qx][kx] * B[qy][ky];
          dphi[a][1] = B[qx][kx] * G[qy][ky];
        }
      double xq[3], J[3][2];
      for (int i = 0; i < 3; i++) {
        xq[i] = Xq[i * nq + Q];
        for (int j = 0; j < 2; j++) J[i][j] = Jq[(j * 3 + i) * nq + Q];
      }
      double cr[3] = {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1],
                      J[0][0] * J[1][1] - J[1][0] * J[0][1]};
      double scale = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      Dual<N> u[3], du[3][2];
      for (int i = 0; i < c; i++) {
        double v = 0, g0 = 0, g1 = 0;
        for (int a = 0; a < nd; a++) {
          v += ue[i * nd + a] * phi[a];
          g0 += ue[i * nd + a] * dphi[a][0];
          g1 += ue[i * nd + a] * dphi[a][1];
        }
        u[i] = mk<N>(v);
        u[i].g[i] = 1.0;
        du[i][0] = mk<N>(g0);
        du[i][0].g[c + 2 * i] = 1.0;
        du[i][1] = mk<N>(g1);
        du[i][1].g[c + 2 * i + 1] = 1.0;
      }
      for (int i = c; i < 3; i++) {
        u[i] = mk<N>(0.0);
        du[i][0] = du[i][1] = mk<N>(0.0);
      }
      Dual<N> o[3];
      bqf<Dual<N>>(mat, prm, xq, J, u, du, o);
      for (int i = 0; i < c; i++) o[i] = o[i] * scale;
      if (mode == 0) {
        for (int i = 0; i < c; i++)
          for (int a = 0; a < nd; a++) out[i * nd + a] += w * o[i].v * phi[a];
      } else if (mode == 1) {
        double din[N];
        for (int i = 0; i < c; i++) {
          double v = 0, g0 = 0, g1 = 0;
          for (int a = 0; a < nd; a++) {
            v += due[i * nd + a] * phi[a];
            g0 += due[i * nd + a] * dphi[a][0];
            g1 += due[i * nd + a] * dphi[a][1];
          }
          din[i] = v;
          din[c + 2 * i] = g0;
          din[c + 2 * i + 1] = g1;
        }
        for (int i = 0; i < c; i++) {
          double acc = 0;
          for (int s = 0; s < N; s++) acc += o[i].g[s] * din[s];
          for (int a = 0; a < nd; a++) out[i * nd + a] += w * acc * phi[a];
        }
      } else {
        for (int jc = 0; jc < c; jc++)
          for (int bb = 0; bb < nd; bb++) {
            double* col = out + size_t(jc * nd + bb) * size_t(ndof);
            for (int ic = 0; ic < c; ic++) {
              double acc = o[ic].g[jc] * phi[bb] + o[ic].g[c + 2 * jc] * dphi[bb][0] + o[ic].g[c + 2 * jc + 1] * dphi[bb][1];
              for (int a = 0; a < nd; a++) col[ic * nd + a] += w * acc * phi[a];
            }
          }
      }
    }
}

}  // namespace

extern "C" {

// Positions and Jacobians at the Gauss points of trilinear hexahedra.
// Xe: [ne][3][8] lexicographic vertex coordinates.  Out: Xq [ne][3][nq],
// Jq [ne][3 (xi)][3 (x)][nq] (geometric_factors.cpp:17-60 layout).
int orc_geometric_factors(int Q, int ne, const double* Xe, double* Xq, double* Jq) {
  if (Q < 1 || Q > 4) return -1;
  const double* pts = gl_points(Q);
  const int nq = Q * Q * Q;
  for (int e = 0; e < ne; e++) {
    const double* X = Xe + size_t(e) * 24;
    for (int qz = 0; qz < Q; qz++)
      for (int qy = 0; qy < Q; qy++)
        for (int qx = 0; qx < Q; qx++) {
          int q = (qz * Q + qy) * Q + qx;
          double s[3] = {pts[qx], pts[qy], pts[qz]};
          double x[3] = {0, 0, 0}, J[3][3] = {};
          for (int v = 0; v < 8; v++) {
            int b[3] = {v & 1, (v >> 1) & 1, (v >> 2) & 1};
            double N[3], dN[3];
            for (int d = 0; d < 3; d++) {
              N[d] = b[d] ? s[d] : 1.0 - s[d];
              dN[d] = b[d] ? 1.0 : -1.0;
            }
            double phi = N[0] * N[1] * N[2];
            double g[3] = {dN[0] * N[1] * N[2], N[0] * dN[1] * N[2], N[0] * N[1] * dN[2]};
            for (int i = 0; i < 3; i++) {
              x[i] += X[i * 8 + v] * phi;
              for (int j = 0; j < 3; j++) J[i][j] += X[i * 8 + v] * g[j];
            }
          }
          for (int i = 0; i < 3; i++) {
            Xq[(size_t(e) * 3 + size_t(i)) * nq + size_t(q)] = x[i];
            for (int j = 0; j < 3; j++) Jq[((size_t(e) * 3 + size_t(j)) * 3 + size_t(i)) * nq + size_t(q)] = J[i][j];
          }
        }
  }
  return 0;
}

// Same for bilinear quadrilateral faces. Xf: [nf][3][4].  Jq [nf][2][3][nq].
int orc_face_geometric_factors(int Q, int nf, const double* Xf, double* Xq, double* Jq) {
  if (Q < 1 || Q > 4) return -1;
  const double* pts = gl_points(Q);
  const int nq = Q * Q;
  for (int e = 0; e < nf; e++) {
    const double* X = Xf + size_t(e) * 12;
    for (int qy = 0; qy < Q; qy++)
      for (int qx = 0; qx < Q; qx++) {
        int q = qy * Q + qx;
        double s[2] = {pts[qx], pts[qy]};
        double x[3] = {0, 0, 0}, J[3][2] = {};
        for (int v = 0; v < 4; v++) {
          int b[2] = {v & 1, (v >> 1) & 1};
          double N[2], dN[2];
          for (int d = 0; d < 2; d++) {
            N[d] = b[d] ? s[d] : 1.0 - s[d];
            dN[d] = b[d] ? 1.0 : -1.0;
          }
          for (int i = 0; i < 3; i++) {
            x[i] += X[i * 4 + v] * N[0] * N[1];
            J[i][0] += X[i * 4 + v] * dN[0] * N[1];
            J[i][1] += X[i * 4 + v] * N[0] * dN[1];
          }
        }
        for (int i = 0; i < 3; i++) {
          Xq[(size_t(e) * 3 + size_t(i)) * nq + size_t(q)] = x[i];
          for (int j = 0; j < 2; j++) Jq[((size_t(e) * 2 + size_t(j)) * 3 + size_t(i)) * nq + size_t(q)] = J[i][j];
        }
      }
  }
  return 0;
}

// Element kernels on E-vectors ([e][comp][node]).  mode 0: residual (J2
// state committed when update != 0); mode 1: Jacobian action at uE on duE;
// mode 2: K_e [e][trial vdof][test vdof].  params: per-element material
// parameters (HEAT {k,f}; NEOHOOKEAN {K,G}; J2 {E,nu,sigma_y,H};
// NONLINEAR_HEAT {k0,beta,f}).  nthreads > 1 runs the element loop on that
// many OpenMP threads (elements are independent; results are identical).
int orc_domain(int mat, int p, int mode, int ne, double t, const double* params, const double* uE, const double* duE,
               const double* Xq, const double* Jq, double* state, int update, double* out, int nthreads) {
  if (p < 1 || p > 3 || mode < 0 || mode > 2) return -1;
  if (mat < 0 || mat > 5) return -1;
  const int c = components_of(mat);
  const int np = params_of(mat);
  Basis3 b(p);
  const int nd = b.nd, nq = b.nq, ndof = nd * c;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int e = 0; e < ne; e++) {
    const double* prm = params ? params + size_t(e) * size_t(np) : nullptr;
    J2State* st = (mat == MAT_J2 && state) ? reinterpret_cast<J2State*>(state) + size_t(e) * size_t(nq) : nullptr;
    J2State zero_state[64];
    if (mat == MAT_J2 && !state) {
      std::memset(zero_state, 0, sizeof(zero_state));
      st = zero_state;
    }
    const double* ue = uE + size_t(e) * ndof;
    const double* due = duE ? duE + size_t(e) * ndof : nullptr;
    const double* X = Xq + size_t(e) * 3 * nq;
    const double* J = Jq + size_t(e) * 9 * nq;
    double* o = out + (mode == 2 ? size_t(e) * ndof * ndof : size_t(e) * ndof);
    if (c == 1) domain_element<1>(mat, p, mode, t, prm, b, ue, due, X, J, st, update != 0, o);
    else domain_element<3>(mat, p, mode, t, prm, b, ue, due, X, J, st, update != 0, o);
  }
  return 0;
}

}  // extern "C"

// ------------------------------------------------------ multi-field domain
// ParameterizedNeoHookeanSolid (parameterized_solid_material.hpp:68-110) in
// SolidMechanics' material integrand with an acceleration field
// (solid_mechanics.hpp:809-850): arguments (u 3, a 3, dK 1, dG 1), per-element
// parameters {density, K0, G0}; source = density a, flux = sigma F^{-T} det F
// with sigma = (lambda ln J I + G (B - I)) / J, K = K0 + dK, G = G0 + dG.
// The derivative with respect to one argument is taken by full forward-mode
// duals over that argument's inputs (values, parent gradients).

constexpr int MAT_PARAM_NEOHOOKEAN = 16;

template <typename S>
void qf_param_neohookean(const double* prm, const S (*grad_u)[3], const S* acc, const S& dK, const S& dG, S* src,
                         S (*flux)[3]) {
  const double rho = prm[0], K0 = prm[1], G0 = prm[2];
  S K = dK + K0, G = dG + G0;
  S lambda = K - G * (2.0 / 3.0);
  M3<S> H;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) H.a[i][j] = grad_u[i][j];
  M3<S> BmI;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      S hh = Z<S>();
      for (int k = 0; k < 3; k++) hh = hh + H.a[i][k] * H.a[j][k];
      BmI.a[i][j] = hh + H.a[j][i] + H.a[i][j];
    }
  S Jm1 = det_ap_im1(H);
  S Jd = Jm1 + 1.0;
  S lg = log1p(Jm1);
  M3<S> F = H;
  for (int i = 0; i < 3; i++) F.a[i][i] = F.a[i][i] + 1.0;
  M3<S> Fi = inv3(F);
  S dF = det3(F);
  for (int i = 0; i < 3; i++) {
    src[i] = acc[i] * rho;
    for (int j = 0; j < 3; j++) {
      S acc_ij = Z<S>();
      for (int k = 0; k < 3; k++) {
        S sig = (lambda * lg * (i == k ? 1.0 : 0.0) + G * BmI.a[i][k]) / Jd;
        acc_ij = acc_ij + sig * Fi.a[j][k];
      }
      flux[i][j] = acc_ij * dF;
    }
  }
}

// values and physical gradients of the four arguments at point q; the
// argument `wrt` (>= 0) carries duals of width N seeded on its inputs
template <int N>
struct MultiPoint {
  Dual<N> gu[3][3], a[3], dK, dG;
};

template <int N>
void multi_point(int wrt, const Basis3& b, int q, const double* const* fe, const M3<double>& Ji, MultiPoint<N>& mp) {
  const int nd = b.nd;
  const int comps[4] = {3, 3, 1, 1};
  const double* phi = &b.phi[size_t(q * nd)];
  const double* dphi = &b.dphi[size_t(q * nd * 3)];
  Dual<N> val[4][3], gpar[4][3][3];
  for (int f = 0; f < 4; f++)
    for (int c = 0; c < comps[f]; c++) {
      double v = 0.0, g[3] = {0, 0, 0};
      for (int a = 0; a < nd; a++) {
        const double x = fe[f][c * nd + a];
        v += x * phi[a];
        for (int j = 0; j < 3; j++) g[j] += x * dphi[a * 3 + j];
      }
      val[f][c] = mk<N>(v);
      if (f == wrt) val[f][c].g[c] = 1.0;
      for (int j = 0; j < 3; j++) {
        gpar[f][c][j] = mk<N>(g[j]);
        if (f == wrt) gpar[f][c][j].g[comps[f] + 3 * c + j] = 1.0;
      }
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      Dual<N> s = mk<N>(0.0);
      for (int k = 0; k < 3; k++) s = s + gpar[0][i][k] * Ji.a[k][j];
      mp.gu[i][j] = s;
    }
  for (int i = 0; i < 3; i++) mp.a[i] = val[1][i];
  mp.dK = val[2][0];
  mp.dG = val[3][0];
}

// one element: mode 0 residual, 1 Jv wrt, 2 K_e wrt ([trial][test]), 3 J^T v wrt
template <int N>
void multi_element(int mode, int wrt, const double* prm, const Basis3& b, const double* const* fe, const double* dE,
                   const double* Xq, const double* Jq, double* out) {
  const int nd = b.nd, nq = b.nq;
  const int cw = N / 4;
  const int test_dofs = 3 * nd;
  if (mode == 0 || mode == 1) std::memset(out, 0, sizeof(double) * size_t(test_dofs));
  if (mode == 2) std::memset(out, 0, sizeof(double) * size_t(cw * nd) * size_t(test_dofs));
  if (mode == 3) std::memset(out, 0, sizeof(double) * size_t(cw * nd));
  (void)Xq;
  for (int q = 0; q < nq; q++) {
    M3<double> Jm;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Jm.a[i][j] = Jq[(j * 3 + i) * nq + q];
    M3<double> Ji = inv3(Jm);
    const double dv = det3(Jm), w = b.w[size_t(q)];
    MultiPoint<N> mp;
    multi_point<N>(mode == 0 ? -1 : wrt, b, q, fe, Ji, mp);
    Dual<N> src[3], flux[3][3];
    qf_param_neohookean<Dual<N>>(prm, mp.gu, mp.a, mp.dK, mp.dG, src, flux);
    // parent-space outputs [source 3][flux 3 x 3] with det J folded in: value and derivative
    double outv[12], D[12][N];
    for (int i = 0; i < 3; i++) {
      Dual<N> sv = src[i] * dv;
      outv[i] = sv.v;
      for (int n = 0; n < N; n++) D[i][n] = sv.g[n];
      for (int k = 0; k < 3; k++) {
        Dual<N> acc = mk<N>(0.0);
        for (int m = 0; m < 3; m++) acc = acc + flux[i][m] * Ji.a[k][m];
        acc = acc * dv;
        outv[3 + 3 * i + k] = acc.v;
        for (int n = 0; n < N; n++) D[3 + 3 * i + k][n] = acc.g[n];
      }
    }
    const double* phi = &b.phi[size_t(q * nd)];
    const double* dphi = &b.dphi[size_t(q * nd * 3)];
    auto integrate_test = [&](const double* o, double* dst) {
      for (int i = 0; i < 3; i++)
        for (int a = 0; a < nd; a++)
          dst[i * nd + a] += w * (o[i] * phi[a] + o[3 + 3 * i] * dphi[a * 3] + o[3 + 3 * i + 1] * dphi[a * 3 + 1] +
                                  o[3 + 3 * i + 2] * dphi[a * 3 + 2]);
    };
    if (mode == 0) {
      integrate_test(outv, out);
      continue;
    }
    if (mode == 1 || mode == 2) {
      const int ncol = mode == 1 ? 1 : cw * nd;
      for (int col = 0; col < ncol; col++) {
        double din[N];
        for (int i = 0; i < N; i++) din[i] = 0.0;
        if (mode == 1) {
          for (int c = 0; c < cw; c++)
            for (int a = 0; a < nd; a++) {
              const double da = dE[c * nd + a];
              din[c] += da * phi[a];
              for (int j = 0; j < 3; j++) din[cw + 3 * c + j] += da * dphi[a * 3 + j];
            }
        } else {
          const int c = col / nd, a = col % nd;
          din[c] = phi[a];
          for (int j = 0; j < 3; j++) din[cw + 3 * c + j] = dphi[a * 3 + j];
        }
        double dout[12];
        for (int r = 0; r < 12; r++) {
          double acc = 0.0;
          for (int k = 0; k < N; k++) acc += D[r][k] * din[k];
          dout[r] = acc;
        }
        integrate_test(dout, mode == 1 ? out : out + size_t(col) * size_t(test_dofs));
      }
      continue;
    }
    // mode 3: v on the test side, D^T, integrated on field wrt
    double vin[12];
    for (int r = 0; r < 12; r++) vin[r] = 0.0;
    for (int i = 0; i < 3; i++)
      for (int a = 0; a < nd; a++) {
        const double va = dE[i * nd + a];
        vin[i] += va * phi[a];
        for (int j = 0; j < 3; j++) vin[3 + 3 * i + j] += va * dphi[a * 3 + j];
      }
    for (int c = 0; c < cw; c++) {
      double s0 = 0.0, g[3] = {0, 0, 0};
      for (int r = 0; r < 12; r++) {
        s0 += D[r][c] * vin[r];
        for (int j = 0; j < 3; j++) g[j] += D[r][cw + 3 * c + j] * vin[r];
      }
      for (int a = 0; a < nd; a++)
        out[c * nd + a] += w * (s0 * phi[a] + g[0] * dphi[a * 3] + g[1] * dphi[a * 3 + 1] + g[2] * dphi[a * 3 + 2]);
    }
  }
}

extern "C" {

// Multi-field material MAT_PARAM_NEOHOOKEAN on E-vectors: uE, aE [e][3][nd],
// kE, gE [e][1][nd]; mode 0 residual -> out [e][3][nd]; 1 Jv with respect to
// argument wrt (dE: that field's E-vector) -> [e][3][nd]; 2 K_e with respect
// to wrt -> [e][cw nd][3 nd]; 3 J^T v (dE: test-space E-vector) -> [e][cw][nd].
int orc_domain_multi(int mat, int p, int mode, int wrt, int ne, double t, const double* params, const double* uE,
                     const double* aE, const double* kE, const double* gE, const double* dE, const double* Xq,
                     const double* Jq, double* out, int nthreads) {
  (void)t;
  if (mat != MAT_PARAM_NEOHOOKEAN || p < 1 || p > 3 || mode < 0 || mode > 3) return -1;
  if (mode > 0 && (wrt < 0 || wrt > 3)) return -1;
  Basis3 b(p);
  const int nd = b.nd, nq = b.nq;
  const int comps[4] = {3, 3, 1, 1};
  const int cw = mode == 0 ? 3 : comps[wrt];
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int e = 0; e < ne; e++) {
    const double* fe[4] = {uE + size_t(e) * 3 * nd, aE + size_t(e) * 3 * nd, kE + size_t(e) * nd, gE + size_t(e) * nd};
    const double* prm = params + size_t(e) * 3;
    const double* X = Xq + size_t(e) * 3 * nq;
    const double* J = Jq + size_t(e) * 9 * nq;
    const double* d = nullptr;
    double* o = nullptr;
    if (mode == 0) o = out + size_t(e) * 3 * nd;
    if (mode == 1) {
      d = dE + size_t(e) * cw * nd;
      o = out + size_t(e) * 3 * nd;
    }
    if (mode == 2) o = out + size_t(e) * size_t(cw * nd) * size_t(3 * nd);
    if (mode == 3) {
      d = dE + size_t(e) * 3 * nd;
      o = out + size_t(e) * cw * nd;
    }
    if (cw == 3) multi_element<12>(mode, wrt, prm, b, fe, d, X, J, o);
    else multi_element<4>(mode, wrt, prm, b, fe, d, X, J, o);
  }
  return 0;
}

// Boundary-face kernels on face E-vectors ([f][comp][node], node
// lexicographic on the face).  params: HEAT_FLUX {q0,q1,alpha}; TRACTION
// {t0[3], t1[3]}; PRESSURE {p}.
int orc_boundary(int mat, int p, int mode, int nf, double t, const double* params, const double* uF, const double* duF,
                 const double* Xq, const double* Jq, double* out) {
  (void)t;
  if (p < 1 || p > 3 || mode < 0 || mode > 2 || mat < 0 || mat > 2) return -1;
  const int c = (mat == BMAT_HEAT_FLUX) ? 1 : 3;
  const int nd = (p + 1) * (p + 1), nq = nd, ndof = nd * c;
  for (int e = 0; e < nf; e++) {
    const double* ue = uF + size_t(e) * ndof;
    const double* due = duF ? duF + size_t(e) * ndof : nullptr;
    const double* X = Xq + size_t(e) * 3 * nq;
    const double* J = Jq + size_t(e) * 6 * nq;
    double* o = out + (mode == 2 ? size_t(e) * ndof * ndof : size_t(e) * ndof);
    if (c == 1) boundary_face<1>(mat, p, mode, params, ue, due, X, J, o);
    else boundary_face<3>(mat, p, mode, params, ue, due, X, J, o);
  }
  return 0;
}


// ---------------------------------------------------------------------------
// Stored-derivative Jacobian action, the way serac applies a linearisation:
// the q-function derivative D is computed once per quadrature point
// (evaluation_kernel_impl with differentiation, domain_integral_kernels.hpp:
// 152-220, D stored after physical->parent at :209-214) and every Jv then
// runs interpolate(du) -> D . du -> integrate with sum factorisation
// (action_of_gradient_kernel, domain_integral_kernels.hpp:277-304;
// hexahedron_H1.inl:169-280).  This is the CPU baseline path.

// D: [e][q][N][N], N = 4c, quadrature weight not included.
int orc_linearize(int mat, int p, int ne, double t, const double* params, const double* uE, const double* Xq,
                  const double* Jq, const double* state, double* D, int nthreads) {
  (void)t;
  if (p < 1 || p > 3 || mat < 0 || mat > 5) return -1;
  const int c = components_of(mat);
  const int np = params_of(mat);
  Basis3 b(p);
  const int nd = b.nd, nq = b.nq, N = 4 * c;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int e = 0; e < ne; e++) {
    const double* prm = params ? params + size_t(e) * size_t(np) : nullptr;
    const double* ue = uE + size_t(e) * nd * c;
    for (int q = 0; q < nq; q++) {
      const double* phi = &b.phi[size_t(q * nd)];
      const double* dphi = &b.dphi[size_t(q * nd * 3)];
      double uval[3] = {0, 0, 0}, ugrad[3][3] = {};
      for (int i = 0; i < c; i++)
        for (int a = 0; a < nd; a++) {
          double ua = ue[i * nd + a];
          uval[i] += ua * phi[a];
          for (int j = 0; j < 3; j++) ugrad[i][j] += ua * dphi[a * 3 + j];
        }
      double J[3][3], xq[3];
      for (int i = 0; i < 3; i++) {
        xq[i] = Xq[(size_t(e) * 3 + i) * nq + q];
        for (int j = 0; j < 3; j++) J[i][j] = Jq[((size_t(e) * 3 + j) * 3 + i) * nq + q];
      }
      J2State st{};
      J2State* sp = nullptr;
      if (mat == MAT_J2) {
        if (state) std::memcpy(&st, state + (size_t(e) * nq + q) * 10, sizeof(J2State));
        sp = &st;
      }
      double vals[12];
      double* Dq = D + (size_t(e) * nq + q) * size_t(N * N);
      if (c == 1) qp_linearise<1>(mat, prm, sp, xq, J, uval, ugrad, vals, Dq);
      else qp_linearise<3>(mat, prm, sp, xq, J, uval, ugrad, vals, Dq);
    }
  }
  return 0;
}

}  // extern "C"

template <int n, int c>
static void apply_linearization_element(const double (&B)[4][4], const double (&G)[4][4], const double (&Bw)[4][4],
                                        const double (&Gw)[4][4], const double* D, const double* due, double* out) {
  constexpr int q = n, nq = q * q * q, N = 4 * c;
  double din[nq][N];
  // interpolate each component (A10/A11, A20/A21/A22, value/gradients)
  for (int i = 0; i < c; i++) {
    const double* X = due + i * n * n * n;  // X[dz][dy][dx]
    double A10[n][n][q], A11[n][n][q];
    for (int dz = 0; dz < n; dz++)
      for (int dy = 0; dy < n; dy++)
        for (int qx = 0; qx < q; qx++) {
          double s0 = 0, s1 = 0;
          for (int dx = 0; dx < n; dx++) {
            double v = X[(dz * n + dy) * n + dx];
            s0 += B[qx][dx] * v;
            s1 += G[qx][dx] * v;
          }
          A10[dz][dy][qx] = s0;
          A11[dz][dy][qx] = s1;
        }
    double A20[n][q][q], A21[n][q][q], A22[n][q][q];
    for (int dz = 0; dz < n; dz++)
      for (int qy = 0; qy < q; qy++)
        for (int qx = 0; qx < q; qx++) {
          double s0 = 0, s1 = 0, s2 = 0;
          for (int dy = 0; dy < n; dy++) {
            s0 += B[qy][dy] * A10[dz][dy][qx];
            s1 += B[qy][dy] * A11[dz][dy][qx];
            s2 += G[qy][dy] * A10[dz][dy][qx];
          }
          A20[dz][qy][qx] = s0;
          A21[dz][qy][qx] = s1;
          A22[dz][qy][qx] = s2;
        }
    for (int qz = 0; qz < q; qz++)
      for (int qy = 0; qy < q; qy++)
        for (int qx = 0; qx < q; qx++) {
          double v = 0, g0 = 0, g1 = 0, g2 = 0;
          for (int dz = 0; dz < n; dz++) {
            v += B[qz][dz] * A20[dz][qy][qx];
            g0 += B[qz][dz] * A21[dz][qy][qx];
            g1 += B[qz][dz] * A22[dz][qy][qx];
            g2 += G[qz][dz] * A20[dz][qy][qx];
          }
          int Q = (qz * q + qy) * q + qx;
          din[Q][i] = v;
          din[Q][c + 3 * i + 0] = g0;
          din[Q][c + 3 * i + 1] = g1;
          din[Q][c + 3 * i + 2] = g2;
        }
  }
  // chain rule
  double dout[nq][N];
  for (int Q = 0; Q < nq; Q++) {
    const double* Dq = D + size_t(Q) * N * N;
    for (int r = 0; r < N; r++) {
      double acc = 0;
      for (int s2 = 0; s2 < N; s2++) acc += Dq[r * N + s2] * din[Q][s2];
      dout[Q][r] = acc;
    }
  }
  // integrate each component with the weighted 1-D matrices
  for (int i = 0; i < c; i++) {
    double A20[q][q][n], A21[q][q][n], A22[q][q][n];
    for (int qz = 0; qz < q; qz++)
      for (int qy = 0; qy < q; qy++)
        for (int dx = 0; dx < n; dx++) {
          double s0 = 0, s1 = 0, s2 = 0;
          for (int qx = 0; qx < q; qx++) {
            int Q = (qz * q + qy) * q + qx;
            s0 += Bw[qx][dx] * dout[Q][i] + Gw[qx][dx] * dout[Q][c + 3 * i];
            s1 += Bw[qx][dx] * dout[Q][c + 3 * i + 1];
            s2 += Bw[qx][dx] * dout[Q][c + 3 * i + 2];
          }
          A20[qz][qy][dx] = s0;
          A21[qz][qy][dx] = s1;
          A22[qz][qy][dx] = s2;
        }
    double A10[q][n][n], A11[q][n][n];
    for (int qz = 0; qz < q; qz++)
      for (int dy = 0; dy < n; dy++)
        for (int dx = 0; dx < n; dx++) {
          double s0 = 0, s1 = 0;
          for (int qy = 0; qy < q; qy++) {
            s0 += Bw[qy][dy] * A20[qz][qy][dx] + Gw[qy][dy] * A21[qz][qy][dx];
            s1 += Bw[qy][dy] * A22[qz][qy][dx];
          }
          A10[qz][dy][dx] = s0;
          A11[qz][dy][dx] = s1;
        }
    for (int dz = 0; dz < n; dz++)
      for (int dy = 0; dy < n; dy++)
        for (int dx = 0; dx < n; dx++) {
          double s0 = 0;
          for (int qz = 0; qz < q; qz++) s0 += Bw[qz][dz] * A10[qz][dy][dx] + Gw[qz][dz] * A11[qz][dy][dx];
          out[i * n * n * n + (dz * n + dy) * n + dx] = s0;
        }
  }
}

extern "C" {

// out E-vector = J(u) duE using the stored derivatives D of orc_linearize.
int orc_apply_linearization(int p, int c, int ne, const double* D, const double* duE, double* out, int nthreads) {
  if (p < 1 || p > 3 || (c != 1 && c != 3)) return -1;
  const int n = p + 1, q = p + 1;
  const double* pts = gl_points(q);
  const double* wts = gl_weights(q);
  double B[4][4] = {}, G[4][4] = {}, Bw[4][4] = {}, Gw[4][4] = {};
  for (int i = 0; i < q; i++) {
    lagrange(n, pts[i], B[i], G[i]);
    for (int k = 0; k < n; k++) {
      Bw[i][k] = B[i][k] * wts[i];
      Gw[i][k] = G[i][k] * wts[i];
    }
  }
  const int nd = n * n * n * c, nq = q * q * q, N = 4 * c;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int e = 0; e < ne; e++) {
    const double* De = D + size_t(e) * nq * N * N;
    const double* de = duE + size_t(e) * nd;
    double* o = out + size_t(e) * nd;
    if (p == 1 && c == 1) apply_linearization_element<2, 1>(B, G, Bw, Gw, De, de, o);
    else if (p == 1 && c == 3) apply_linearization_element<2, 3>(B, G, Bw, Gw, De, de, o);
    else if (p == 2 && c == 1) apply_linearization_element<3, 1>(B, G, Bw, Gw, De, de, o);
    else if (p == 2 && c == 3) apply_linearization_element<3, 3>(B, G, Bw, Gw, De, de, o);
    else if (p == 3 && c == 1) apply_linearization_element<4, 1>(B, G, Bw, Gw, De, de, o);
    else apply_linearization_element<4, 3>(B, G, Bw, Gw, De, de, o);
  }
  return 0;
}

// E[(e c + k) npe + j] = L[k nnodes + conn[e npe + j]]   (element_restriction.cpp:443-454)
int orc_gather(int64_t ne, int npe, int c, int64_t nnodes, const int64_t* conn, const double* L, double* E,
               int nthreads) {
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int64_t e = 0; e < ne; e++)
    for (int k = 0; k < c; k++)
      for (int j = 0; j < npe; j++) E[(e * c + k) * npe + j] = L[k * nnodes + conn[e * npe + j]];
  return 0;
}

// L[k nnodes + n] = sum over the node's (element, local) entries of E, in
// entry order (the node-owner form of ScatterAdd, element_restriction.cpp:456-467)
int orc_scatter(int64_t nnodes, int npe, int c, const int64_t* node_ptr, const int64_t* node_ent, const double* E,
                double* L, int nthreads) {
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int64_t nd = 0; nd < nnodes; nd++)
    for (int k = 0; k < c; k++) {
      double acc = 0.0;
      for (int64_t i = node_ptr[nd]; i < node_ptr[nd + 1]; i++) {
        int64_t ent = node_ent[i];
        int64_t e = ent / npe, j = ent % npe;
        acc += E[(e * c + k) * npe + j];
      }
      L[k * nnodes + nd] = acc;
    }
  return 0;
}

}  // extern "C"
