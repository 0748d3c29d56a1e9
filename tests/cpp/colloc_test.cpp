// Host check of the collocated sum factorisation used by the residual and
// Jacobian-action kernels (include/sfx/quadrature.hpp): the Gauss-point
// derivative matrix D[q][j] = l_j'(x_q) equals G B^-1, so differentiating a
// field's point values (B along x, y, z, then D along one direction) gives
// the parent gradient that B and G give directly, and the transposed
// (integration) form agrees too.  Orders 1-3.  Built with g++ by
// tests/test_colloc_host.py; prints one line per failed check.
#include <cmath>
#include <cstdio>
#include <random>

#include "sfx/quadrature.hpp"

using namespace sfx;

namespace {

int failures = 0;

void expect_close(const char* what, int p, double a, double b, double tol) {
  if (!(std::fabs(a - b) <= tol * std::fmax(1.0, std::fabs(b)))) {
    std::printf("FAIL %s p=%d: %.17g vs %.17g\n", what, p, a, b);
    failures++;
  }
}

template <int P>
void check() {
  constexpr int Q = P + 1;
  constexpr BasisTable<P> T = make_basis_table<P>();
  // D B = G
  for (int q = 0; q < Q; q++)
    for (int k = 0; k < Q; k++) {
      double s = 0;
      for (int j = 0; j < Q; j++) s += T.D[q][j] * T.B[j][k];
      expect_close("D B = G", P, s, T.G[q][k], 1e-13);
    }
  std::mt19937_64 rng(7 + P);
  std::normal_distribution<double> N01;
  double u[Q][Q][Q], f[3][Q][Q][Q];
  for (auto& a : u)
    for (auto& b : a)
      for (double& c : b) c = N01(rng);
  for (auto& d : f)
    for (auto& a : d)
      for (auto& b : a)
        for (double& c : b) c = N01(rng);
  auto basis = [&](int dir, int deriv, int q, int k) { return (dir == deriv) ? T.G[q][k] : T.B[q][k]; };
  // gradient at every point: direct (B, G) and collocated (B^3, then D)
  double w[Q][Q][Q] = {};
  for (int qz = 0; qz < Q; qz++)
    for (int qy = 0; qy < Q; qy++)
      for (int qx = 0; qx < Q; qx++)
        for (int kz = 0; kz < Q; kz++)
          for (int ky = 0; ky < Q; ky++)
            for (int kx = 0; kx < Q; kx++) w[qz][qy][qx] += T.B[qx][kx] * T.B[qy][ky] * T.B[qz][kz] * u[kz][ky][kx];
  for (int d = 0; d < 3; d++)
    for (int qz = 0; qz < Q; qz++)
      for (int qy = 0; qy < Q; qy++)
        for (int qx = 0; qx < Q; qx++) {
          double direct = 0;
          for (int kz = 0; kz < Q; kz++)
            for (int ky = 0; ky < Q; ky++)
              for (int kx = 0; kx < Q; kx++)
                direct += basis(0, d, qx, kx) * basis(1, d, qy, ky) * basis(2, d, qz, kz) * u[kz][ky][kx];
          double colloc = 0;
          for (int j = 0; j < Q; j++) {
            if (d == 0) colloc += T.D[qx][j] * w[qz][qy][j];
            if (d == 1) colloc += T.D[qy][j] * w[qz][j][qx];
            if (d == 2) colloc += T.D[qz][j] * w[j][qy][qx];
          }
          expect_close("gradient", P, colloc, direct, 1e-12);
        }
  // integration of a flux f[d] at the points against the basis gradients:
  // direct r[k] = sum_q sum_d dphi_k/dxi_d(q) f[d](q); collocated: D^T at
  // the points, then B^T along x, y, z
  double t[Q][Q][Q] = {};
  for (int qz = 0; qz < Q; qz++)
    for (int qy = 0; qy < Q; qy++)
      for (int qx = 0; qx < Q; qx++)
        for (int j = 0; j < Q; j++) {
          t[qz][qy][qx] += T.D[j][qx] * f[0][qz][qy][j];
          t[qz][qy][qx] += T.D[j][qy] * f[1][qz][j][qx];
          t[qz][qy][qx] += T.D[j][qz] * f[2][j][qy][qx];
        }
  for (int kz = 0; kz < Q; kz++)
    for (int ky = 0; ky < Q; ky++)
      for (int kx = 0; kx < Q; kx++) {
        double direct = 0, colloc = 0;
        for (int qz = 0; qz < Q; qz++)
          for (int qy = 0; qy < Q; qy++)
            for (int qx = 0; qx < Q; qx++) {
              for (int d = 0; d < 3; d++)
                direct += basis(0, d, qx, kx) * basis(1, d, qy, ky) * basis(2, d, qz, kz) * f[d][qz][qy][qx];
              colloc += T.B[qx][kx] * T.B[qy][ky] * T.B[qz][kz] * t[qz][qy][qx];
            }
        expect_close("integration", P, colloc, direct, 1e-12);
      }
}

}  // namespace

int main() {
  check<1>();
  check<2>();
  check<3>();
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("OK\n");
  return 0;
}
