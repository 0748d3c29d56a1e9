// sfx — 1-D rules and bases for tensor-product H1 elements.
//
// Gauss-Legendre points/weights on [0, 1] use the same tabulated digits as
// serac (numerics/functional/polynomials.hpp:42-52, 271-282) so that both
// codes integrate with identical rules.  Shape functions are the Lagrange
// polynomials on the Gauss-Lobatto nodes of [0, 1] (polynomials.hpp:493-541),
// evaluated here by the product formula.
#pragma once

#include "sfx/tensor.hpp"

namespace sfx {

SFX_HDI constexpr double gl_point(int q, int i) {
  if (q == 1) return 0.5;
  if (q == 2) return i == 0 ? 0.2113248654051871 : 0.7886751345948129;
  if (q == 3) return i == 0 ? 0.1127016653792583 : (i == 1 ? 0.500000000000000 : 0.887298334620742);
  if (q == 4) {
    return i == 0 ? 0.0694318442029737 : (i == 1 ? 0.330009478207572 : (i == 2 ? 0.669990521792428 : 0.930568155797026));
  }
  return 0.0;
}

SFX_HDI constexpr double gl_weight(int q, int i) {
  if (q == 1) return 1.0;
  if (q == 2) return 0.5;
  if (q == 3) return i == 1 ? 0.444444444444444 : 0.277777777777778;
  if (q == 4) return (i == 0 || i == 3) ? 0.173927422568727 : 0.326072577431273;
  return 0.0;
}

SFX_HDI constexpr double gll_node(int n, int k) {
  if (n == 2) return k == 0 ? 0.0 : 1.0;
  if (n == 3) return k == 0 ? 0.0 : (k == 1 ? 0.5 : 1.0);
  if (n == 4) {
    // 1/2 -+ 1/(2 sqrt 5)
    return k == 0 ? 0.0 : (k == 1 ? 0.27639320225002103 : (k == 2 ? 0.72360679774997897 : 1.0));
  }
  return 0.0;
}

/// Lagrange polynomial k on the n Gauss-Lobatto nodes, and its derivative, at x.
SFX_HDI constexpr void gll_basis(int n, int k, double x, double& phi, double& dphi) {
  double v = 1.0, d = 0.0;
  double xk = gll_node(n, k);
  for (int j = 0; j < n; j++) {
    if (j == k) continue;
    double xj = gll_node(n, j);
    double term = (x - xj) / (xk - xj);
    d = d * term + v / (xk - xj);
    v = v * term;
  }
  phi = v;
  dphi = d;
}

/// Derivative at Gauss point i of the Lagrange polynomial j on the n Gauss
/// points (the collocated derivative matrix, equal to G B^-1: a degree n-1
/// field is fixed by its n point values, so differentiating those values is
/// exact).
SFX_HDI constexpr double gl_lagrange_dphi(int n, int i, int j) {
  double v = 1.0, d = 0.0;
  const double x = gl_point(n, i), xj = gl_point(n, j);
  for (int m = 0; m < n; m++) {
    if (m == j) continue;
    const double xm = gl_point(n, m);
    const double term = (x - xm) / (xj - xm);
    d = d * term + v / (xj - xm);
    v = v * term;
  }
  return d;
}

/// B[q][k] = phi_k(x_q), G[q][k] = phi_k'(x_q) on the (p+1)-point rule.
SFX_HDI constexpr double basis_B(int p, int q, int k) {
  double phi = 0, dphi = 0;
  gll_basis(p + 1, k, gl_point(p + 1, q), phi, dphi);
  return phi;
}
SFX_HDI constexpr double basis_G(int p, int q, int k) {
  double phi = 0, dphi = 0;
  gll_basis(p + 1, k, gl_point(p + 1, q), phi, dphi);
  return dphi;
}

/// B and G of the (p+1)-point rule, evaluated at compile time.
template <int P>
struct BasisTable {
  double B[P + 1][P + 1];
  double G[P + 1][P + 1];
  double D[P + 1][P + 1];  // collocated derivative at the Gauss points, D[q][j] = l_j'(x_q)
};

template <int P>
constexpr BasisTable<P> make_basis_table() {
  BasisTable<P> t{};
  for (int q = 0; q <= P; q++)
    for (int k = 0; k <= P; k++) {
      double phi = 0, dphi = 0;
      gll_basis(P + 1, k, gl_point(P + 1, q), phi, dphi);
      t.B[q][k] = phi;
      t.G[q][k] = dphi;
      t.D[q][k] = gl_lagrange_dphi(P + 1, q, k);
    }
  return t;
}

#if defined(__CUDACC__)
/// Device copies of the tables (constant memory, no runtime FP64 work).
static __constant__ BasisTable<1> kBasis1 = make_basis_table<1>();
static __constant__ BasisTable<2> kBasis2 = make_basis_table<2>();
static __constant__ BasisTable<3> kBasis3 = make_basis_table<3>();
template <int P>
__device__ inline const BasisTable<P>& basis_table();
template <>
__device__ inline const BasisTable<1>& basis_table<1>() { return kBasis1; }
template <>
__device__ inline const BasisTable<2>& basis_table<2>() { return kBasis2; }
template <>
__device__ inline const BasisTable<3>& basis_table<3>() { return kBasis3; }
#endif

}  // namespace sfx
