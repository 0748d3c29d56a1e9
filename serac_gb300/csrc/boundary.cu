// Boundary integrals over the sides of the structured box
// (serac: Functional::AddBoundaryIntegral, functional.hpp:328-354;
// boundary_integral_kernels.hpp:112-325; face restriction, element_restriction.cpp:279-388).
//
// Faces of side s are parametrised (s, t) so that dX/ds x dX/dt points out of
// the box; faces are numbered t-major within a side, sides in increasing
// order; face-local node ks + (p+1) kt.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "dispatch.hpp"
#include "form.hpp"
#include "graph.hpp"
#include "sfx.h"
#include "sfx/boundary.cuh"
#include "sfx/materials.hpp"
#include "sfx/sensitivity.cuh"

using namespace sfx_impl;

namespace {

using namespace sfx;

struct Side {
  int axis, hi, s_axis, t_axis;
};
// side -> (fixed axis, fixed at max?, s axis, t axis); outward normal = J_s x J_t
constexpr Side kSides[7] = {{0, 0, 0, 0}, {2, 0, 1, 0}, {1, 0, 0, 2}, {0, 1, 1, 2},
                            {1, 1, 2, 0}, {0, 0, 2, 1}, {2, 1, 0, 1}};

template <typename Fn>
int visit_bmaterial(const BoundaryIntegral& bi, Fn&& fn) {
  const auto& p = bi.params;
  switch (bi.material) {
    case SFX_BMAT_HEAT_FLUX:
      return fn.template operator()<1>(boundary_models::HeatFlux{p[0], p[1], p[2]});
    case SFX_BMAT_TRACTION: {
      boundary_models::Traction q{};
      for (int i = 0; i < 3; i++) {
        q.t0[i] = p[size_t(i)];
        q.t1[i] = p[size_t(3 + i)];
      }
      return fn.template operator()<3>(q);
    }
    case SFX_BMAT_PRESSURE: return fn.template operator()<3>(boundary_models::Pressure{p[0]});
  }
  return fail(SFX_ERR_UNSUPPORTED, "unknown boundary material");
}

int bmaterial_info(int material, int* components, int* nparams) {
  switch (material) {
    case SFX_BMAT_HEAT_FLUX: *components = 1; *nparams = 3; return SFX_OK;
    case SFX_BMAT_TRACTION: *components = 3; *nparams = 6; return SFX_OK;
    case SFX_BMAT_PRESSURE: *components = 3; *nparams = 1; return SFX_OK;
  }
  return fail(SFX_ERR_UNSUPPORTED, "unknown boundary material id");
}

template <int P, int MODE, typename Real>
struct FaceFn {
  const sfx_form_s& f;
  const BoundaryIntegral& bi;
  const Real* u;
  const Real* du;
  Real* out;
  double t;
  cudaStream_t s;
  template <int C, typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1);
    constexpr int FPW = 32 / NQ;
    if (bi.num_faces == 0) return SFX_OK;
    Real* E = std::is_same<Real, double>::value ? reinterpret_cast<Real*>(f.ef64.p) : reinterpret_cast<Real*>(f.ef32.p);
    kernels::FaceArgs<Real> a{u, du, E, bi.fconn.p, bi.fgeom.p, f.nnodes, bi.num_faces, t};
    const int64_t warps = (bi.num_faces + FPW - 1) / FPW;
    kernels::face_kernel<P, C, MODE, Real, QF><<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(a, qf);
    kernels::face_scatter_kernel<C, NQ, Real><<<unsigned((bi.num_face_nodes + 255) / 256), 256, 0, s>>>(
        E, bi.node_ptr.p, bi.node_ids.p, bi.node_ent.p, out, bi.num_face_nodes, f.nnodes);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("face kernel launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

template <int P, typename Real>
struct FaceTransposeFn {
  const sfx_form_s& f;
  const BoundaryIntegral& bi;
  const Real* u;
  const Real* v;
  Real* out;
  cudaStream_t s;
  template <int C, typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1);
    constexpr int FPW = 32 / NQ;
    if (bi.num_faces == 0) return SFX_OK;
    Real* E = std::is_same<Real, double>::value ? reinterpret_cast<Real*>(f.ef64.p) : reinterpret_cast<Real*>(f.ef32.p);
    kernels::FaceArgs<Real> a{u, v, E, bi.fconn.p, bi.fgeom.p, f.nnodes, bi.num_faces, f.t_lin};
    const int64_t warps = (bi.num_faces + FPW - 1) / FPW;
    kernels::face_jvp_transpose_kernel<P, C, Real, QF><<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(a, qf);
    kernels::face_scatter_kernel<C, NQ, Real><<<unsigned((bi.num_face_nodes + 255) / 256), 256, 0, s>>>(
        E, bi.node_ptr.p, bi.node_ids.p, bi.node_ent.p, out, bi.num_face_nodes, f.nnodes);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess)
      return fail(SFX_ERR_CUDA, std::string("transposed face kernel launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

template <int P>
struct FaceMatrixFn {
  sfx_form_s& f;
  const BoundaryIntegral& bi;
  double* values;  // CSR values (accumulate) or nullptr
  double* diag;    // diagonal (accumulate) or nullptr
  cudaStream_t s;
  template <int C, typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1);
    constexpr int FPW = 32 / NQ;
    constexpr int NDOF = C * NQ;
    if (bi.num_faces == 0) return SFX_OK;
    const size_t need = size_t(bi.num_faces) * NDOF * NDOF;
    if (f.kf.n < need && f.kf.alloc(need) != cudaSuccess) return fail(SFX_ERR_NOMEM, "face matrix scratch");
    kernels::FaceArgs<double> a{f.u_lin64.p, nullptr, f.kf.p, bi.fconn.p, bi.fgeom.p, f.nnodes, bi.num_faces, f.t_lin};
    const int64_t warps = (bi.num_faces + FPW - 1) / FPW;
    kernels::face_matrix_kernel<P, C, QF><<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(a, qf);
    if (values) {
      with_graph(f, [&](auto g) {
        kernels::face_csr_kernel<P, C><<<unsigned((bi.num_face_nodes * C + 127) / 128), 128, 0, s>>>(
            g, f.row_ptr.p, bi.fconn.p, bi.node_ptr.p, bi.node_ids.p, bi.node_ent.p, f.kf.p, values,
            bi.num_face_nodes);
        return SFX_OK;
      });
    }
    if (diag) {
      kernels::face_diag_kernel<C, NQ><<<unsigned((bi.num_face_nodes + 255) / 256), 256, 0, s>>>(
          bi.node_ptr.p, bi.node_ids.p, bi.node_ent.p, f.kf.p, diag, bi.num_face_nodes, f.nnodes);
    }
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("face matrix launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

}  // namespace

namespace sfx_impl {

template <int P>
struct ShapeFaceFn {
  const sfx_form_s& f;
  const BoundaryIntegral& bi;
  const double* u;
  const double* dshape;
  double* out;
  double t;
  cudaStream_t s;
  template <int C, typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1);
    constexpr int FPW = 32 / NQ;
    if (bi.num_faces == 0) return SFX_OK;
    kernels::FaceArgs<double> a{u, nullptr, f.ef64.p, bi.fconn.p, bi.fgeom.p, f.nnodes, bi.num_faces, t};
    const int64_t warps = (bi.num_faces + FPW - 1) / FPW;
    kernels::face_shape_jvp_kernel<P, C, QF><<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(
        a, qf, bi.Xf.p, f.has_shape ? f.shape.p : nullptr, dshape);
    kernels::face_scatter_kernel<C, NQ, double><<<unsigned((bi.num_face_nodes + 255) / 256), 256, 0, s>>>(
        f.ef64.p, bi.node_ptr.p, bi.node_ids.p, bi.node_ent.p, out, bi.num_face_nodes, f.nnodes);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("face shape jvp launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

template <int P>
struct ShapeFaceVjpFn {
  const sfx_form_s& f;
  const BoundaryIntegral& bi;
  const double* u;
  const double* lam;
  double* out;
  double t;
  cudaStream_t s;
  template <int C, typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1);
    constexpr int FPW = 32 / NQ;
    if (bi.num_faces == 0) return SFX_OK;
    kernels::FaceArgs<double> a{u, nullptr, f.efshape.p, bi.fconn.p, bi.fgeom.p, f.nnodes, bi.num_faces, t};
    const int64_t warps = (bi.num_faces + FPW - 1) / FPW;
    kernels::face_shape_adjoint_kernel<P, C, kernels::SHAPE_VJP, QF><<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(
        a, qf, bi.Xf.p, f.has_shape ? f.shape.p : nullptr, lam);
    kernels::face_scatter_kernel<3, NQ, double><<<unsigned((bi.num_face_nodes + 255) / 256), 256, 0, s>>>(
        f.efshape.p, bi.node_ptr.p, bi.node_ids.p, bi.node_ent.p, out, bi.num_face_nodes, f.nnodes);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("face shape vjp launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

// out += (d(boundary residual)/dp)^T lam for every boundary integral of the form
int launch_boundary_shape_vjp(const sfx_form_s& f, const double* u, const double* lam, double* out, double t,
                              cudaStream_t s) {
  for (const auto& bi : f.boundary) {
    const int rc = f.p == 1 ? visit_bmaterial(bi, ShapeFaceVjpFn<1>{f, bi, u, lam, out, t, s})
                            : visit_bmaterial(bi, ShapeFaceVjpFn<2>{f, bi, u, lam, out, t, s});
    if (rc) return rc;
  }
  return SFX_OK;
}

// out += d(boundary residual)/dp dshape for every boundary integral of the form
int launch_boundary_shape_jvp(const sfx_form_s& f, const double* u, const double* dshape, double* out, double t,
                              cudaStream_t s) {
  for (const auto& bi : f.boundary) {
    const int rc = f.p == 1 ? visit_bmaterial(bi, ShapeFaceFn<1>{f, bi, u, dshape, out, t, s})
                            : visit_bmaterial(bi, ShapeFaceFn<2>{f, bi, u, dshape, out, t, s});
    if (rc) return rc;
  }
  return SFX_OK;
}

int launch_boundary(const sfx_form_s& f, int mode, const double* u, const double* du, double* out, double t,
                    cudaStream_t s) {
  for (const auto& bi : f.boundary) {
    int rc = SFX_OK;
    if (mode == 2) {
      rc = f.p == 1 ? visit_bmaterial(bi, FaceFn<1, kernels::JVP, double>{f, bi, u, du, out, t, s})
                    : visit_bmaterial(bi, FaceFn<2, kernels::JVP, double>{f, bi, u, du, out, t, s});
    } else {
      rc = f.p == 1 ? visit_bmaterial(bi, FaceFn<1, kernels::RESIDUAL, double>{f, bi, u, du, out, t, s})
                    : visit_bmaterial(bi, FaceFn<2, kernels::RESIDUAL, double>{f, bi, u, du, out, t, s});
    }
    if (rc) return rc;
  }
  return SFX_OK;
}

int launch_boundary_jvp_f32(const sfx_form_s& f, const float* u, const float* du, float* out, double t,
                            cudaStream_t s) {
  for (const auto& bi : f.boundary) {
    int rc = f.p == 1 ? visit_bmaterial(bi, FaceFn<1, kernels::JVP, float>{f, bi, u, du, out, t, s})
                      : visit_bmaterial(bi, FaceFn<2, kernels::JVP, float>{f, bi, u, du, out, t, s});
    if (rc) return rc;
  }
  return SFX_OK;
}

int launch_boundary_transpose(const sfx_form_s& f, const double* v, double* out, cudaStream_t s) {
  for (const auto& bi : f.boundary) {
    const int rc = f.p == 1 ? visit_bmaterial(bi, FaceTransposeFn<1, double>{f, bi, f.u_lin64.p, v, out, s})
                            : visit_bmaterial(bi, FaceTransposeFn<2, double>{f, bi, f.u_lin64.p, v, out, s});
    if (rc) return rc;
  }
  return SFX_OK;
}

int launch_boundary_transpose_f32(const sfx_form_s& f, const float* v, float* out, cudaStream_t s) {
  for (const auto& bi : f.boundary) {
    const int rc = f.p == 1 ? visit_bmaterial(bi, FaceTransposeFn<1, float>{f, bi, f.u_lin32.p, v, out, s})
                            : visit_bmaterial(bi, FaceTransposeFn<2, float>{f, bi, f.u_lin32.p, v, out, s});
    if (rc) return rc;
  }
  return SFX_OK;
}

int compute_face_geometry(sfx_form_s& f, BoundaryIntegral& bi, cudaStream_t s) {
  const int Q = f.p + 1;
  const int64_t nqt = bi.num_faces * Q * Q;
  if (nqt == 0) return SFX_OK;
  const unsigned blocks = unsigned((nqt + 255) / 256);
  if (f.has_shape) {
    if (f.p == 1)
      kernels::face_geometry_shape_kernel<1><<<blocks, 256, 0, s>>>(bi.Xf.p, bi.fconn.p, f.shape.p, f.nnodes,
                                                                    bi.fgeom.p, bi.num_faces);
    else
      kernels::face_geometry_shape_kernel<2><<<blocks, 256, 0, s>>>(bi.Xf.p, bi.fconn.p, f.shape.p, f.nnodes,
                                                                    bi.fgeom.p, bi.num_faces);
  } else {
    if (Q == 2) kernels::face_geometry_kernel<2><<<blocks, 256, 0, s>>>(bi.Xf.p, bi.fgeom.p, bi.num_faces);
    else kernels::face_geometry_kernel<3><<<blocks, 256, 0, s>>>(bi.Xf.p, bi.fgeom.p, bi.num_faces);
  }
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

int assemble_boundary(sfx_form_s& f, double* values, double* diag, cudaStream_t s) {
  for (const auto& bi : f.boundary) {
    int rc = f.p == 1 ? visit_bmaterial(bi, FaceMatrixFn<1>{f, bi, values, diag, s})
                      : visit_bmaterial(bi, FaceMatrixFn<2>{f, bi, values, diag, s});
    if (rc) return rc;
  }
  return SFX_OK;
}

}  // namespace sfx_impl

namespace sfx_impl {
// faces of the sides in side_mask: connectivity (outward (s, t) order), vertex
// coordinates, compact face-node map, geometric factors, face scratch
int finish_faces(sfx_form_s* form, const std::vector<int32_t>& fconn, const std::vector<double>& Xf,
                 BoundaryIntegral& bi);

int build_faces(sfx_form_s* form, int side_mask, BoundaryIntegral& bi) {
  if (form->general)
    return fail(SFX_ERR_INVALID, "side masks need a structured mesh; give faces as (element, side) pairs");
  if (side_mask <= 0 || side_mask >= 64) return fail(SFX_ERR_INVALID, "side mask must select sides 1..6");
  const auto& m = form->mesh;
  const int p = form->p, n = p + 1, npf = n * n;
  const int64_t dims[3] = {m.nx, m.ny, m.nz};
  const int64_t N[3] = {int64_t(p) * m.nx + 1, int64_t(p) * m.ny + 1, int64_t(p) * m.nz + 1};
  std::vector<int32_t> fconn;
  std::vector<double> Xf;
  for (int side = 1; side <= 6; side++) {
    if (!(side_mask & (1 << (side - 1)))) continue;
    const Side sd = kSides[side];
    const int64_t fixed = sd.hi ? dims[sd.axis] : 0;
    for (int64_t ft = 0; ft < dims[sd.t_axis]; ft++)
      for (int64_t fs = 0; fs < dims[sd.s_axis]; fs++) {
        for (int i = 0; i < 3; i++)
          for (int v = 0; v < 4; v++) {
            int64_t idx[3] = {0, 0, 0};
            idx[sd.axis] = fixed;
            idx[sd.s_axis] = fs + (v & 1);
            idx[sd.t_axis] = ft + (v >> 1);
            const int64_t vid = idx[0] + int64_t(m.nx + 1) * (idx[1] + int64_t(m.ny + 1) * idx[2]);
            Xf.push_back(m.vertices[size_t(vid * 3 + i)]);
          }
        for (int kt = 0; kt < n; kt++)
          for (int ks = 0; ks < n; ks++) {
            int64_t idx[3] = {0, 0, 0};
            idx[sd.axis] = p * fixed;
            idx[sd.s_axis] = p * fs + ks;
            idx[sd.t_axis] = p * ft + kt;
            fconn.push_back(int32_t(idx[0] + N[0] * (idx[1] + N[1] * idx[2])));
          }
      }
  }
  return finish_faces(form, fconn, Xf, bi);
}

// faces (element, local side) of an imported element table: the face nodes
// and vertices in the element's own frame, parametrised like the box sides
// (J_s x J_t points out of the element for a positively oriented element)
int build_faces_list(sfx_form_s* form, int64_t n, const int32_t* face_elem, const int32_t* face_side,
                     BoundaryIntegral& bi) {
  if (n > 0 && (!face_elem || !face_side)) return fail(SFX_ERR_INVALID, "null face list");
  if (form->conn_host.empty()) {  // structured form: host copies of its tables, once
    form->conn_host.resize(size_t(form->ne) * form->NPE);
    form->Xe_host.resize(size_t(form->ne) * 24);
    SFX_CUDA_TRY(cudaMemcpy(form->conn_host.data(), form->conn.p, form->conn_host.size() * sizeof(int32_t),
                            cudaMemcpyDeviceToHost));
    SFX_CUDA_TRY(cudaMemcpy(form->Xe_host.data(), form->Xe.p, form->Xe_host.size() * sizeof(double),
                            cudaMemcpyDeviceToHost));
  }
  const int p = form->p, nn1 = p + 1;
  std::vector<int32_t> fconn;
  std::vector<double> Xf;
  fconn.reserve(size_t(n) * nn1 * nn1);
  Xf.reserve(size_t(n) * 12);
  for (int64_t k = 0; k < n; k++) {
    const int64_t e = face_elem[k];
    const int side = face_side[k];
    if (e < 0 || e >= form->ne) return fail(SFX_ERR_INVALID, "face element out of range");
    if (side < 1 || side > 6) return fail(SFX_ERR_INVALID, "face side must be 1..6");
    const Side sd = kSides[side];
    for (int i = 0; i < 3; i++)
      for (int v = 0; v < 4; v++) {
        int b[3] = {0, 0, 0};
        b[sd.axis] = sd.hi;
        b[sd.s_axis] = v & 1;
        b[sd.t_axis] = v >> 1;
        const int corner = b[0] + 2 * b[1] + 4 * b[2];
        Xf.push_back(form->Xe_host[size_t(e * 24 + i * 8 + corner)]);
      }
    for (int kt = 0; kt < nn1; kt++)
      for (int ks = 0; ks < nn1; ks++) {
        int idx[3] = {0, 0, 0};
        idx[sd.axis] = sd.hi ? p : 0;
        idx[sd.s_axis] = ks;
        idx[sd.t_axis] = kt;
        const int local = idx[0] + nn1 * (idx[1] + nn1 * idx[2]);
        fconn.push_back(form->conn_host[size_t(e * form->NPE + local)]);
      }
  }
  return finish_faces(form, fconn, Xf, bi);
}

// compact face-node map, device tables, geometric factors and face scratch of
// the faces fconn [f][(p+1)^2] with vertices Xf [f][3][4]
int finish_faces(sfx_form_s* form, const std::vector<int32_t>& fconn, const std::vector<double>& Xf,
                 BoundaryIntegral& bi) {
  const int p = form->p, npf = (p + 1) * (p + 1);
  bi.num_faces = int64_t(fconn.size()) / npf;
  // compact face-node map: distinct nodes ascending, entries in face order
  std::vector<int32_t> order(fconn.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = int32_t(i);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return fconn[size_t(a)] < fconn[size_t(b)]; });
  std::vector<int32_t> ids, ptr{0}, ent;
  for (size_t k = 0; k < order.size(); k++) {
    const int32_t nd = fconn[size_t(order[k])];
    if (ids.empty() || ids.back() != nd) {
      if (!ids.empty()) ptr.push_back(int32_t(ent.size()));
      ids.push_back(nd);
    }
    ent.push_back(order[k]);
  }
  ptr.push_back(int32_t(ent.size()));
  bi.num_face_nodes = int64_t(ids.size());
  const int Q = p + 1, nq = Q * Q;
  const int64_t nqt = bi.num_faces * nq;
  cudaError_t err;
  if ((err = bi.fconn.upload(fconn.data(), fconn.size())) != cudaSuccess ||
      (err = bi.node_ptr.upload(ptr.data(), ptr.size())) != cudaSuccess ||
      (err = bi.node_ids.upload(ids.data(), ids.size())) != cudaSuccess ||
      (err = bi.node_ent.upload(ent.data(), ent.size())) != cudaSuccess ||
      (err = bi.Xf.upload(Xf.data(), Xf.size())) != cudaSuccess ||
      (err = bi.fgeom.alloc(size_t(nqt) * kernels::FGEOM_STRIDE)) != cudaSuccess)
    return fail(SFX_ERR_CUDA, std::string("boundary setup: ") + cudaGetErrorString(err));
  if (int rc = compute_face_geometry(*form, bi, nullptr)) return rc;
  if ((err = cudaDeviceSynchronize()) != cudaSuccess)
    return fail(SFX_ERR_CUDA, std::string("face geometry: ") + cudaGetErrorString(err));
  const size_t escr = size_t(bi.num_faces) * npf * form->c;
  if (form->ef64.n < escr) {
    if (form->ef64.alloc(escr) != cudaSuccess || form->ef32.alloc(escr) != cudaSuccess)
      return fail(SFX_ERR_NOMEM, "face scratch allocation");
  }
  return SFX_OK;
}
}  // namespace sfx_impl

extern "C" int sfx_form_add_boundary_integral(sfx_form form, int bmaterial, int side_mask, const double* params) {
  if (!form) return fail(SFX_ERR_INVALID, "null form");
  int comps = 0, np = 0;
  if (int rc = bmaterial_info(bmaterial, &comps, &np)) return rc;
  if (comps != form->c) return fail(SFX_ERR_INVALID, "boundary material component count does not match the space");
  if (form->qoi) return fail(SFX_ERR_INVALID, "a quantity of interest takes sfx_qoi_add_boundary_integral");
  if (!params) return fail(SFX_ERR_INVALID, "null parameters");
  BoundaryIntegral bi;
  bi.material = bmaterial;
  bi.params.assign(params, params + np);
  if (int rc = build_faces(form, side_mask, bi)) return rc;
  form->boundary.push_back(std::move(bi));
  return SFX_OK;
}

extern "C" int sfx_form_add_boundary_integral_faces(sfx_form form, int bmaterial, int64_t num_faces,
                                                    const int32_t* face_elem, const int32_t* face_side,
                                                    const double* params) {
  if (!form) return fail(SFX_ERR_INVALID, "null form");
  int comps = 0, np = 0;
  if (int rc = bmaterial_info(bmaterial, &comps, &np)) return rc;
  if (comps != form->c) return fail(SFX_ERR_INVALID, "boundary material component count does not match the space");
  if (form->qoi) return fail(SFX_ERR_INVALID, "a quantity of interest takes sfx_qoi_add_boundary_integral_faces");
  if (!params) return fail(SFX_ERR_INVALID, "null parameters");
  BoundaryIntegral bi;
  bi.material = bmaterial;
  bi.params.assign(params, params + np);
  if (int rc = build_faces_list(form, num_faces, face_elem, face_side, bi)) return rc;
  form->boundary.push_back(std::move(bi));
  return SFX_OK;
}

extern "C" int sfx_form_add_face_set_faces(sfx_form form, int64_t num_faces, const int32_t* face_elem,
                                           const int32_t* face_side, int* face_set) {
  if (!form || !face_set) return fail(SFX_ERR_INVALID, "null argument");
  BoundaryIntegral bi;
  bi.material = -1;
  if (int rc = build_faces_list(form, num_faces, face_elem, face_side, bi)) return rc;
  form->face_sets.push_back(std::move(bi));
  *face_set = int(form->face_sets.size()) - 1;
  return SFX_OK;
}

extern "C" int sfx_form_add_face_set(sfx_form form, int side_mask, int* face_set) {
  if (!form || !face_set) return fail(SFX_ERR_INVALID, "null argument");
  BoundaryIntegral bi;
  bi.material = -1;  // evaluated by the caller's kernels
  if (int rc = build_faces(form, side_mask, bi)) return rc;
  form->face_sets.push_back(std::move(bi));
  *face_set = int(form->face_sets.size()) - 1;
  return SFX_OK;
}

extern "C" int sfx_form_get_face_layout(sfx_form form, int face_set, sfx_face_layout* out) {
  if (!form || !out) return fail(SFX_ERR_INVALID, "null argument");
  if (face_set < 0 || size_t(face_set) >= form->face_sets.size()) return fail(SFX_ERR_INVALID, "no such face set");
  const BoundaryIntegral& bi = form->face_sets[size_t(face_set)];
  sfx_face_layout L{};
  L.num_faces = bi.num_faces;
  L.nodes_per_face = (form->p + 1) * (form->p + 1);
  L.fconn = bi.fconn.p;
  L.fgeom = bi.fgeom.p;
  L.num_face_nodes = bi.num_face_nodes;
  L.node_ptr = bi.node_ptr.p;
  L.node_ids = bi.node_ids.p;
  L.node_ent = bi.node_ent.p;
  L.face_vertices = bi.Xf.p;
  *out = L;
  return SFX_OK;
}
