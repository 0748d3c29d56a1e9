// Test driver for the header-only C++ front-end (include/sfx/functional.hpp):
// user-written q-function objects, instantiated in this translation unit,
// through Functional<H1<p,c>(H1<p,c>)>.  Built into a shared library by
// tests/test_gpu_frontend.py and called through ctypes; host arrays in/out.
#include <cuda_runtime.h>

#include <type_traits>
#include <vector>

#include "sfx/functional.hpp"
#include "sfx/materials.hpp"

namespace {

// a user q-function: linear scalar model with every derivative block populated
struct UserThermal {
  template <typename X, typename T>
  SFX_HD auto operator()(double, const X& position, const T& temperature) const {
    using namespace sfx;
    auto x = get<0>(position);
    auto u = get<0>(temperature);
    auto g = get<1>(temperature);
    tensor<double, 3> d01{{0.0, 1.0, 2.0}}, d10{{0.0, 2.0, 8.0}};
    tensor<double, 3, 3> d11{};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) d11[i][j] = double(i + j * (j + 1) + 1);
    auto source = 1.0 * u + dot(d01, g) + 0.5 * x[0] * x[1];
    auto flux = u * d10 + dot(d11, g);
    return tuple{source, flux};
  }
};

// a user q-function: compressible Neo-Hookean written out by hand
struct UserNeoHookean {
  double K, G;
  template <typename X, typename D>
  SFX_HD auto operator()(double, const X&, const D& displacement) const {
    using namespace sfx;
    auto H = get<1>(displacement);
    auto F = H + Identity<3>();
    auto J = det(F);
    auto B = dot(F, transpose(F));
    double lambda = K - (2.0 / 3.0) * G;
    using std::log;
    auto sigma = (lambda * log(J) * Identity<3>() + G * (B - Identity<3>())) / J;
    return tuple{zero{}, dot(sigma, transpose(inv(F))) * J};
  }
};

// user boundary q-functions: a follower pressure along the deformed normal per
// unit reference area, and a heat flux with a Robin term
struct UserPressure {
  double p;
  template <typename X, typename D>
  SFX_HD auto operator()(double, const X& position, const D& displacement) const {
    using namespace sfx;
    auto n = cross(get<1>(position) + get<1>(displacement));
    return p * (n / norm(cross(get<1>(position))));
  }
};
struct UserFlux {
  double q0, q1, alpha;
  template <typename X, typename T>
  SFX_HD auto operator()(double, const X& position, const T& temperature) const {
    using namespace sfx;
    return -1.0 * (alpha * get<0>(temperature) + (q0 + q1 * get<0>(position)[0]));
  }
};

using J2 = sfx::solid_mechanics::J2SmallStrain<sfx::solid_mechanics::LinearHardening>;

template <typename F>
void copy_out(const double* dev, double* host, size_t n) {
  cudaMemcpy(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost);
}

struct Buffers {
  double *u, *du, *r, *jv, *diag;
  float *du32, *jv32;
  size_t n;
  Buffers(size_t n_) : n(n_) {
    cudaMalloc(&u, n * 8);
    cudaMalloc(&du, n * 8);
    cudaMalloc(&r, n * 8);
    cudaMalloc(&jv, n * 8);
    cudaMalloc(&diag, n * 8);
    cudaMalloc(&du32, n * 4);
    cudaMalloc(&jv32, n * 4);
  }
  ~Buffers() {
    cudaFree(u);
    cudaFree(du);
    cudaFree(r);
    cudaFree(jv);
    cudaFree(diag);
    cudaFree(du32);
    cudaFree(jv32);
  }
};

// outputs: residual, residual at linearisation, jv, jv (FP32, as double), diagonal, CSR values
template <typename FunctionalT, typename Setup>
int run_on(const sfx::Mesh& mesh, const double* u, const double* du, double* out_r, double* out_r2, double* out_jv,
           double* out_jv32, double* out_diag, double* out_csr, int64_t* out_nnz, Setup&& setup) {
  try {
    FunctionalT f(mesh);
    setup(f);
    const size_t n = size_t(f.num_dofs());
    Buffers b(n);
    cudaMemcpy(b.u, u, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(b.du, du, n * 8, cudaMemcpyHostToDevice);
    std::vector<float> du32(du, du + n);
    cudaMemcpy(b.du32, du32.data(), n * 4, cudaMemcpyHostToDevice);
    const double* r = f(0.0, b.u);
    cudaMemcpy(out_r, r, n * 8, cudaMemcpyDeviceToHost);
    auto [r2, grad] = f(0.0, sfx::differentiate_wrt(b.u));
    cudaMemcpy(out_r2, r2, n * 8, cudaMemcpyDeviceToHost);
    grad.Mult(b.du, b.jv);
    cudaMemcpy(out_jv, b.jv, n * 8, cudaMemcpyDeviceToHost);
    grad.MultF32(b.du32, b.jv32);
    std::vector<float> jv32(n);
    cudaMemcpy(jv32.data(), b.jv32, n * 4, cudaMemcpyDeviceToHost);
    for (size_t i = 0; i < n; i++) out_jv32[i] = jv32[i];
    grad.AssembleDiagonal(b.diag);
    cudaMemcpy(out_diag, b.diag, n * 8, cudaMemcpyDeviceToHost);
    sfx::CSRMatrix A = assemble(grad);
    if (out_csr) cudaMemcpy(out_csr, A.values->p, size_t(A.nnz) * 8, cudaMemcpyDeviceToHost);
    *out_nnz = A.nnz;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
  } catch (const std::exception&) {
    return -1;
  }
}

template <typename FunctionalT, typename Setup>
int run(int nx, int ny, int nz, const double* V, const double* u, const double* du, double* out_r, double* out_r2,
        double* out_jv, double* out_jv32, double* out_diag, double* out_csr, int64_t* out_nnz, Setup&& setup) {
  try {
    auto mesh = sfx::Mesh::StructuredHex(nx, ny, nz, V);
    return run_on<FunctionalT>(mesh, u, du, out_r, out_r2, out_jv, out_jv32, out_diag, out_csr, out_nnz, setup);
  } catch (const std::exception&) {
    return -1;
  }
}

}  // namespace

extern "C" int frontend_thermal(int p, int nx, int ny, int nz, const double* V, const double* u, const double* du,
                                double* r, double* r2, double* jv, double* jv32, double* diag, double* csr,
                                int64_t* nnz) {
  auto setup = [](auto& f) { f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserThermal{}); };
  if (p == 1)
    return run<sfx::Functional<sfx::H1<1, 1>(sfx::H1<1, 1>)>>(nx, ny, nz, V, u, du, r, r2, jv, jv32, diag, csr, nnz,
                                                              setup);
  return run<sfx::Functional<sfx::H1<2, 1>(sfx::H1<2, 1>)>>(nx, ny, nz, V, u, du, r, r2, jv, jv32, diag, csr, nnz,
                                                            setup);
}

extern "C" int frontend_neohookean(int p, double K, double G, int nx, int ny, int nz, const double* V, const double* u,
                                   const double* du, double* r, double* r2, double* jv, double* jv32, double* diag,
                                   double* csr, int64_t* nnz) {
  auto setup = [K, G](auto& f) { f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserNeoHookean{K, G}); };
  if (p == 1)
    return run<sfx::Functional<sfx::H1<1, 3>(sfx::H1<1, 3>)>>(nx, ny, nz, V, u, du, r, r2, jv, jv32, diag, csr, nnz,
                                                              setup);
  return run<sfx::Functional<sfx::H1<2, 3>(sfx::H1<2, 3>)>>(nx, ny, nz, V, u, du, r, r2, jv, jv32, diag, csr, nnz,
                                                            setup);
}

// Neo-Hookean with a user follower-pressure boundary integral on sides in side_mask
extern "C" int frontend_neohookean_pressure(double K, double G, double pressure, int side_mask, int nx, int ny, int nz,
                                            const double* V, const double* u, const double* du, double* r, double* r2,
                                            double* jv, double* jv32, double* diag, double* csr, int64_t* nnz) {
  auto setup = [=](auto& f) {
    f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserNeoHookean{K, G});
    f.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserPressure{pressure}, side_mask);
  };
  return run<sfx::Functional<sfx::H1<2, 3>(sfx::H1<2, 3>)>>(nx, ny, nz, V, u, du, r, r2, jv, jv32, diag, csr, nnz,
                                                            setup);
}

// the thermal model with a user heat-flux boundary integral
extern "C" int frontend_thermal_flux(int p, double q0, double q1, double alpha, int side_mask, int nx, int ny, int nz,
                                     const double* V, const double* u, const double* du, double* r, double* r2,
                                     double* jv, double* jv32, double* diag, double* csr, int64_t* nnz) {
  auto setup = [=](auto& f) {
    f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserThermal{});
    f.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserFlux{q0, q1, alpha}, side_mask);
  };
  if (p == 1)
    return run<sfx::Functional<sfx::H1<1, 1>(sfx::H1<1, 1>)>>(nx, ny, nz, V, u, du, r, r2, jv, jv32, diag, csr, nnz,
                                                              setup);
  return run<sfx::Functional<sfx::H1<2, 1>(sfx::H1<2, 1>)>>(nx, ny, nz, V, u, du, r, r2, jv, jv32, diag, csr, nnz,
                                                            setup);
}

// Neo-Hookean on a shape-displaced configuration (ShapeAwareFunctional)
extern "C" int frontend_neohookean_shape(double K, double G, int nx, int ny, int nz, const double* V,
                                         const double* shape_host, int64_t nshape, const double* u, const double* du,
                                         double* r, double* r2, double* jv, double* jv32, double* diag, double* csr,
                                         int64_t* nnz) {
  double* shape = nullptr;
  if (cudaMalloc(&shape, size_t(nshape) * 8) != cudaSuccess) return -2;
  cudaMemcpy(shape, shape_host, size_t(nshape) * 8, cudaMemcpyHostToDevice);
  auto setup = [K, G, shape](auto& f) {
    f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserNeoHookean{K, G});
    f.SetShapeDisplacement(shape);
  };
  const int rc = run<sfx::ShapeAwareFunctional<sfx::H1<2, 3>, sfx::H1<2, 3>(sfx::H1<2, 3>)>>(
      nx, ny, nz, V, u, du, r, r2, jv, jv32, diag, csr, nnz, setup);
  cudaFree(shape);
  return rc;
}

// J2 through the library's material functor with a QuadratureData state:
// commit the state at u (updateQdata), then linearise at 1.5 u.
extern "C" int frontend_j2(int nx, int ny, int nz, const double* V, const double* u, const double* du, double E,
                           double nu, double sy, double H, double* r_commit, double* state_out, double* r, double* jv) {
  try {
    auto mesh = sfx::Mesh::StructuredHex(nx, ny, nz, V);
    sfx::Functional<sfx::H1<1, 3>(sfx::H1<1, 3>)> f(mesh);
    J2 mat{};
    mat.E = E;
    mat.nu = nu;
    mat.hardening = sfx::solid_mechanics::LinearHardening{sy, H};
    auto qdata = std::make_shared<sfx::QuadratureData<J2::State>>(f.num_elements(), f.points_per_element);
    f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{},
                        sfx::solid_mechanics::MaterialStressFunctor<J2, false>{mat}, qdata);
    const size_t n = size_t(f.num_dofs());
    Buffers b(n);
    cudaMemcpy(b.u, u, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(b.du, du, n * 8, cudaMemcpyHostToDevice);
    f.updateQdata(true);
    f.residual(0.0, b.u, b.r);
    f.updateQdata(false);
    cudaMemcpy(r_commit, b.r, n * 8, cudaMemcpyDeviceToHost);
    const int64_t npts = qdata->num_points();
    std::vector<double> soa(size_t(npts) * 10);
    cudaMemcpy(soa.data(), qdata->device(), soa.size() * 8, cudaMemcpyDeviceToHost);
    for (int64_t q = 0; q < npts; q++)
      for (int k = 0; k < 10; k++) state_out[q * 10 + k] = soa[size_t(k * npts + q)];
    std::vector<double> u15(u, u + n);
    for (auto& x : u15) x *= 1.5;
    cudaMemcpy(b.u, u15.data(), n * 8, cudaMemcpyHostToDevice);
    auto [rr, grad] = f(0.0, sfx::differentiate_wrt(b.u));
    cudaMemcpy(r, rr, n * 8, cudaMemcpyDeviceToHost);
    grad.Mult(b.du, b.jv);
    cudaMemcpy(jv, b.jv, n * 8, cudaMemcpyDeviceToHost);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
  } catch (const std::exception&) {
    return -1;
  }
}

namespace {

// user QoI integrands (scalar field): X0^2 + sin X1 + X0 u^3 + (1 + X2)/2 |grad u|^2
// on the domain and X0 - X1 + cos(u X1) + (du/ds)^2 / 4 on faces
struct UserPolyQoI {
  template <typename X, typename T>
  SFX_HD auto operator()(double, const X& position, const T& temperature) const {
    using namespace sfx;
    using std::sin;
    auto x = get<0>(position);
    auto u = get<0>(temperature);
    auto g = get<1>(temperature);
    return x[0] * x[0] + sin(x[1]) + x[0] * u * u * u + 0.5 * (1.0 + x[2]) * dot(g, g);
  }
};
struct UserPolyFaceQoI {
  template <typename X, typename T>
  SFX_HD auto operator()(double, const X& position, const T& temperature) const {
    using namespace sfx;
    using std::cos;
    auto x = get<0>(position);
    auto u = get<0>(temperature);
    auto g = get<1>(temperature);
    return x[0] - x[1] + cos(u * x[1]) + 0.25 * g[0] * g[0];
  }
};
// user QoI integrands (vector field): Neo-Hookean stored energy written from
// F = I + H, and the normal displacement u . n on faces
struct UserEnergyQoI {
  double K, G;
  template <typename X, typename D>
  SFX_HD auto operator()(double, const X&, const D& displacement) const {
    using namespace sfx;
    using std::log;
    auto H = get<1>(displacement);
    auto F = H + Identity<3>();
    auto lnJ = log(det(F));
    auto trC = F[0][0] * F[0][0];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        if (i + j > 0) trC = trC + F[i][j] * F[i][j];
    double lambda = K - (2.0 / 3.0) * G;
    return 0.5 * G * (trC - 3.0) - G * lnJ + 0.5 * lambda * lnJ * lnJ;
  }
};
struct UserNormalQoI {
  template <typename X, typename D>
  SFX_HD auto operator()(double, const X& position, const D& displacement) const {
    using namespace sfx;
    auto n = cross(get<1>(position));
    return dot(get<0>(displacement), n / norm(n));
  }
};

template <typename QoIT, typename Setup>
int run_qoi(int nx, int ny, int nz, const double* V, const double* u, const double* du, double* value,
            double* value2, double* action, double* grad, Setup&& setup) {
  try {
    auto mesh = sfx::Mesh::StructuredHex(nx, ny, nz, V);
    QoIT q(mesh);
    setup(q);
    const size_t n = size_t(q.num_dofs());
    Buffers b(n);
    cudaMemcpy(b.u, u, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(b.du, du, n * 8, cudaMemcpyHostToDevice);
    *value = q(0.0, b.u);
    auto [v2, g] = q(0.0, sfx::differentiate_wrt(b.u));
    *value2 = v2;
    *action = g(b.du);
    const double* gv = assemble(g);
    cudaMemcpy(grad, gv, n * 8, cudaMemcpyDeviceToHost);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
  } catch (const std::exception&) {
    return -1;
  }
}

}  // namespace

// scalar QoI: the polynomial integrand on the domain and on the sides in side_mask
extern "C" int frontend_qoi_poly(int p, int side_mask, int nx, int ny, int nz, const double* V, const double* u,
                                 const double* du, double* value, double* value2, double* action, double* grad) {
  auto setup = [=](auto& q) {
    q.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserPolyQoI{});
    q.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserPolyFaceQoI{}, side_mask);
  };
  if (p == 1)
    return run_qoi<sfx::Functional<double(sfx::H1<1, 1>)>>(nx, ny, nz, V, u, du, value, value2, action, grad, setup);
  return run_qoi<sfx::Functional<double(sfx::H1<2, 1>)>>(nx, ny, nz, V, u, du, value, value2, action, grad, setup);
}

// vector QoI: stored energy on the domain plus u . n on the sides in side_mask (Q2)
extern "C" int frontend_qoi_energy(double K, double G, int side_mask, int nx, int ny, int nz, const double* V,
                                   const double* u, const double* du, double* value, double* value2, double* action,
                                   double* grad) {
  auto setup = [=](auto& q) {
    q.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserEnergyQoI{K, G});
    q.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserNormalQoI{}, side_mask);
  };
  return run_qoi<sfx::Functional<double(sfx::H1<2, 3>)>>(nx, ny, nz, V, u, du, value, value2, action, grad, setup);
}

// transposed actions of the user Neo-Hookean + follower pressure functional (Q2)
extern "C" int frontend_neohookean_pressure_transpose(double K, double G, double pressure, int side_mask, int nx,
                                                      int ny, int nz, const double* V, const double* u,
                                                      const double* v, double* jt, double* jt32) {
  try {
    auto mesh = sfx::Mesh::StructuredHex(nx, ny, nz, V);
    sfx::Functional<sfx::H1<2, 3>(sfx::H1<2, 3>)> f(mesh);
    f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserNeoHookean{K, G});
    f.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserPressure{pressure}, side_mask);
    const size_t n = size_t(f.num_dofs());
    Buffers b(n);
    cudaMemcpy(b.u, u, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(b.du, v, n * 8, cudaMemcpyHostToDevice);
    std::vector<float> v32(v, v + n);
    cudaMemcpy(b.du32, v32.data(), n * 4, cudaMemcpyHostToDevice);
    auto [r, grad] = f(0.0, sfx::differentiate_wrt(b.u));
    (void)r;
    grad.MultTranspose(b.du, b.jv);
    cudaMemcpy(jt, b.jv, n * 8, cudaMemcpyDeviceToHost);
    grad.MultTransposeF32(b.du32, b.jv32);
    std::vector<float> out32(n);
    cudaMemcpy(out32.data(), b.jv32, n * 4, cudaMemcpyDeviceToHost);
    for (size_t i = 0; i < n; i++) jt32[i] = out32[i];
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
  } catch (const std::exception&) {
    return -1;
  }
}

// Neo-Hookean with a user follower pressure over a face list, on an imported
// element table (Q2): residual, linearisation, actions, diagonal and CSR
extern "C" int frontend_table_neohookean_pressure(double K, double G, double pressure, int64_t ne, int64_t nn,
                                                  const int32_t* table, const double* corners, int64_t nf,
                                                  const int32_t* face_elem, const int32_t* face_side, const double* u,
                                                  const double* du, double* r, double* r2, double* jv, double* jv32,
                                                  double* diag, double* csr, int64_t* nnz) {
  try {
    auto mesh = sfx::Mesh::FromTable(2, ne, nn, table, corners);
    std::vector<int32_t> fe(face_elem, face_elem + nf), fs(face_side, face_side + nf);
    auto setup = [&](auto& f) {
      f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserNeoHookean{K, G});
      f.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserPressure{pressure}, fe, fs);
    };
    return run_on<sfx::Functional<sfx::H1<2, 3>(sfx::H1<2, 3>)>>(mesh, u, du, r, r2, jv, jv32, diag, csr, nnz, setup);
  } catch (const std::exception&) {
    return -1;
  }
}

// scalar QoI (user domain and face integrands) on an imported element table
extern "C" int frontend_table_qoi_poly(int p, int64_t ne, int64_t nn, const int32_t* table, const double* corners,
                                       int64_t nf, const int32_t* face_elem, const int32_t* face_side, const double* u,
                                       const double* du, double* value, double* value2, double* action,
                                       double* grad) {
  try {
    auto mesh = sfx::Mesh::FromTable(p, ne, nn, table, corners);
    std::vector<int32_t> fe(face_elem, face_elem + nf), fs(face_side, face_side + nf);
    auto setup = [&](auto& q) {
      q.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserPolyQoI{});
      q.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserPolyFaceQoI{}, fe, fs);
    };
    auto go = [&](auto order) -> int {
      using QoIT = sfx::Functional<double(sfx::H1<decltype(order)::value, 1>)>;
      QoIT q(mesh);
      setup(q);
      const size_t n = size_t(q.num_dofs());
      Buffers b(n);
      cudaMemcpy(b.u, u, n * 8, cudaMemcpyHostToDevice);
      cudaMemcpy(b.du, du, n * 8, cudaMemcpyHostToDevice);
      *value = q(0.0, b.u);
      auto [v2, g] = q(0.0, sfx::differentiate_wrt(b.u));
      *value2 = v2;
      *action = g(b.du);
      cudaMemcpy(grad, assemble(g), n * 8, cudaMemcpyDeviceToHost);
      return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
    };
    if (p == 1) return go(std::integral_constant<int, 1>{});
    return go(std::integral_constant<int, 2>{});
  } catch (const std::exception&) {
    return -1;
  }
}

// shape derivatives of user q-functions on a shape-displaced configuration:
// dR/dp dshape and (dR/dp)^T lam of Neo-Hookean + follower pressure (Q2), and
// dQ/dp of the user energy + normal-displacement QoI
extern "C" int frontend_shape_sensitivity(double K, double G, double pressure, int side_mask, int nx, int ny, int nz,
                                          const double* V, const double* shape_host, const double* u_host,
                                          const double* dshape_host, const double* lam_host, double* jvp_out,
                                          double* vjp_out, double* qoi_shape_out) {
  try {
    auto mesh = sfx::Mesh::StructuredHex(nx, ny, nz, V);
    sfx::Functional<sfx::H1<2, 3>(sfx::H1<2, 3>)> f(mesh);
    f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserNeoHookean{K, G});
    f.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserPressure{pressure}, side_mask);
    sfx::Functional<double(sfx::H1<2, 3>)> q(mesh);
    q.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, UserEnergyQoI{K, G});
    q.AddBoundaryIntegral(sfx::Dimension<2>{}, sfx::DependsOn<0>{}, UserNormalQoI{}, side_mask);
    const size_t n = size_t(f.num_dofs()), ns = n;  // 3 components: the shape space has as many entries
    double *shape, *u, *dshape, *lam, *a, *b, *c;
    cudaMalloc(&shape, ns * 8);
    cudaMalloc(&u, n * 8);
    cudaMalloc(&dshape, ns * 8);
    cudaMalloc(&lam, n * 8);
    cudaMalloc(&a, n * 8);
    cudaMalloc(&b, ns * 8);
    cudaMalloc(&c, ns * 8);
    cudaMemcpy(shape, shape_host, ns * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(u, u_host, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dshape, dshape_host, ns * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(lam, lam_host, n * 8, cudaMemcpyHostToDevice);
    f.SetShapeDisplacement(shape);
    q.SetShapeDisplacement(shape);
    f.ShapeJvp(0.0, u, dshape, a);
    f.ShapeVjp(0.0, u, lam, b);
    q.ShapeGradient(0.0, u, c);
    cudaMemcpy(jvp_out, a, n * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(vjp_out, b, ns * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(qoi_shape_out, c, ns * 8, cudaMemcpyDeviceToHost);
    for (double* x : {shape, u, dshape, lam, a, b, c}) cudaFree(x);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
  } catch (const std::exception&) {
    return -1;
  }
}

// --------------------------------------------------------------- multi-field
namespace {

// a user q-function of four fields, written out by hand: SolidMechanics'
// material integrand with acceleration and bulk / shear modulus offset fields
// around a compressible Neo-Hookean solid
struct UserParamNeoHookean {
  double rho, K0, G0;
  template <typename X, typename U, typename A, typename PK, typename PG>
  SFX_HD auto operator()(double, const X&, const U& displacement, const A& acceleration, const PK& dK,
                         const PG& dG) const {
    using namespace sfx;
    using std::log1p;
    auto H = get<1>(displacement);
    auto K = K0 + get<0>(dK);
    auto G = G0 + get<0>(dG);
    auto lambda = K - (2.0 / 3.0) * G;
    auto F = H + Identity<3>();
    auto Jm1 = detApIm1(H);
    auto J = Jm1 + 1.0;
    auto BmI = dot(H, transpose(H)) + transpose(H) + H;
    auto sigma = (lambda * log1p(Jm1) * Identity<3>() + G * BmI) / J;
    return tuple{rho * get<0>(acceleration), dot(sigma, transpose(inv(F))) * J};
  }
};

template <int P>
int run_multi(int nx, int ny, int nz, const double* V, const double* const* host_fields, int wrt, const double* d,
              const double* v, double rho, double K0, double G0, double* r, double* jv, double* jt) {
  try {
    auto mesh = sfx::Mesh::StructuredHex(nx, ny, nz, V);
    sfx::Functional<sfx::H1<P, 3>(sfx::H1<P, 3>, sfx::H1<P, 3>, sfx::H1<P, 1>, sfx::H1<P, 1>)> f(mesh);
    f.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0, 1, 2, 3>{}, UserParamNeoHookean{rho, K0, G0});
    const int64_t N = f.num_nodes();
    const int comps[4] = {3, 3, 1, 1};
    sfx::DeviceArray<double> fld[4], dd(size_t(comps[wrt] * N)), vv(size_t(3 * N)), out(size_t(3 * N)),
        outw(size_t(comps[wrt] * N));
    for (int k = 0; k < 4; k++) {
      fld[k].resize(size_t(comps[k] * N));
      cudaMemcpy(fld[k].p, host_fields[k], sizeof(double) * size_t(comps[k] * N), cudaMemcpyHostToDevice);
    }
    cudaMemcpy(dd.p, d, sizeof(double) * size_t(comps[wrt] * N), cudaMemcpyHostToDevice);
    cudaMemcpy(vv.p, v, sizeof(double) * size_t(3 * N), cudaMemcpyHostToDevice);
    const double* R = f(0.0, fld[0].p, fld[1].p, fld[2].p, fld[3].p);
    cudaMemcpy(r, R, sizeof(double) * size_t(3 * N), cudaMemcpyDeviceToHost);
    auto grad_of = [&](auto& self) -> decltype(auto) {
      using sfx::differentiate_wrt;
      switch (wrt) {
        case 0: return std::get<1>(self(0.0, differentiate_wrt(fld[0].p), fld[1].p, fld[2].p, fld[3].p));
        case 1: return std::get<1>(self(0.0, fld[0].p, differentiate_wrt(fld[1].p), fld[2].p, fld[3].p));
        case 2: return std::get<1>(self(0.0, fld[0].p, fld[1].p, differentiate_wrt(fld[2].p), fld[3].p));
        default: return std::get<1>(self(0.0, fld[0].p, fld[1].p, fld[2].p, differentiate_wrt(fld[3].p)));
      }
    };
    auto& J = grad_of(f);
    J.Mult(dd.p, out.p);
    J.MultTranspose(vv.p, outw.p);
    cudaMemcpy(jv, out.p, sizeof(double) * size_t(3 * N), cudaMemcpyDeviceToHost);
    cudaMemcpy(jt, outw.p, sizeof(double) * size_t(comps[wrt] * N), cudaMemcpyDeviceToHost);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
  } catch (const std::exception&) {
    return -1;
  }
}

}  // namespace

// Functional<H1<p,3>(H1<p,3>, H1<p,3>, H1<p,1>, H1<p,1>)> with a user
// q-function under DependsOn<0, 1, 2, 3>: residual, and the derivative with
// respect to field wrt applied to d and, transposed, to v (host arrays)
extern "C" int frontend_multi(int p, int nx, int ny, int nz, const double* V, const double* u, const double* a,
                              const double* dK, const double* dG, int wrt, const double* d, const double* v,
                              double rho, double K0, double G0, double* r, double* jv, double* jt) {
  const double* fields[4] = {u, a, dK, dG};
  if (wrt < 0 || wrt > 3) return -1;
  return p == 1 ? run_multi<1>(nx, ny, nz, V, fields, wrt, d, v, rho, K0, G0, r, jv, jt)
                : run_multi<2>(nx, ny, nz, V, fields, wrt, d, v, rho, K0, G0, r, jv, jt);
}
