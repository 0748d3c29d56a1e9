// Quantities of interest: Functional<double(H1<p,c>)> (functional_qoi.inl:58-528)
// with the built-in integrands of sfx/qoi.cuh, over the whole domain and over
// box sides.  Values and directional derivatives reduce to one device double
// through per-element / per-face sums and a fixed-shape two-pass tree;
// gradients scatter like residuals (node-owner order): deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "dispatch.hpp"
#include "form.hpp"
#include "sfx.h"
#include "sfx/qoi.cuh"
#include "sfx/sensitivity.cuh"

using namespace sfx_impl;

namespace {

using namespace sfx;
constexpr int kMaxQoiPartials = kernels::kQoiMaxPartials;

// number of parameters of a QoI kind for c components, -1 if the kind is not
// available there (boundary: whether the integral is over faces)
int qoi_nparams(int kind, int c, bool boundary) {
  switch (kind) {
    case SFX_QOI_MEASURE: return 0;
    case SFX_QOI_POSITION: return 3;
    case SFX_QOI_FIELD: return c;
    case SFX_QOI_NEOHOOKEAN_ENERGY: return (!boundary && c == 3) ? 2 : -1;
    case SFX_QOI_NORMAL_FIELD: return (boundary && c == 3) ? 0 : -1;
    case SFX_QOI_POLY_TEST: return 0;
  }
  return -1;
}

// Calls fn(qf) with the integrand of a domain QoI integral.
template <int C, typename Fn>
int visit_domain_qoi(const QoiIntegral& qi, Fn&& fn) {
  const auto& p = qi.params;
  switch (qi.kind) {
    case SFX_QOI_MEASURE: return fn(qoi_models::Measure{});
    case SFX_QOI_POSITION: return fn(qoi_models::PositionMoment{{p[0], p[1], p[2]}});
    case SFX_QOI_FIELD: {
      qoi_models::FieldIntegral<C> q{};
      for (int c = 0; c < C; c++) q.w[c] = p[size_t(c)];
      return fn(q);
    }
    case SFX_QOI_NEOHOOKEAN_ENERGY:
      if constexpr (C == 3) return fn(qoi_models::NeoHookeanEnergy{p[0], p[1]});
      break;
    case SFX_QOI_POLY_TEST: return fn(qoi_models::PolyTest<C>{});
  }
  return fail(SFX_ERR_UNSUPPORTED, "QoI kind not available on the domain");
}

template <int C, typename Fn>
int visit_face_qoi(const BoundaryIntegral& bi, Fn&& fn) {
  const auto& p = bi.params;
  switch (bi.material) {
    case SFX_QOI_MEASURE: return fn(qoi_models::Measure{});
    case SFX_QOI_POSITION: return fn(qoi_models::PositionMoment{{p[0], p[1], p[2]}});
    case SFX_QOI_FIELD: {
      qoi_models::FieldIntegral<C> q{};
      for (int c = 0; c < C; c++) q.w[c] = p[size_t(c)];
      return fn(q);
    }
    case SFX_QOI_NORMAL_FIELD:
      if constexpr (C == 3) return fn(qoi_models::NormalField{});
      break;
    case SFX_QOI_POLY_TEST: return fn(qoi_models::PolyTestFace<C>{});
  }
  return fail(SFX_ERR_UNSUPPORTED, "QoI kind not available on faces");
}

template <int P, int C, int MODE>
struct DomainQoiFn {
  const sfx_form_s& f;
  const double* u;
  const double* du;
  double* vals;
  double t;
  cudaStream_t s;
  template <typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
    constexpr int EPW = 32 / NQ;
    if (f.ne == 0) return SFX_OK;
    kernels::DomainArgs<double> a{u, du, f.e64.p, f.conn.p, f.geom64.p, nullptr, nullptr, f.nnodes, f.ne, t};
    const int64_t warps = (f.ne + EPW - 1) / EPW;
    kernels::qoi_domain_kernel<P, C, MODE, QF><<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(a, qf, vals);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("QoI kernel launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

template <int P, int C, int MODE>
struct FaceQoiFn {
  const sfx_form_s& f;
  const BoundaryIntegral& bi;
  const double* u;
  const double* du;
  double* grad;  // accumulated into (QOI_GRADIENT)
  double* vals;
  double t;
  cudaStream_t s;
  template <typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1);
    constexpr int FPW = 32 / NQ;
    if (bi.num_faces == 0) return SFX_OK;
    kernels::FaceArgs<double> a{u, du, f.ef64.p, bi.fconn.p, bi.fgeom.p, f.nnodes, bi.num_faces, t};
    const int64_t warps = (bi.num_faces + FPW - 1) / FPW;
    kernels::qoi_face_kernel<P, C, MODE, QF><<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(a, qf, vals);
    if constexpr (MODE == kernels::QOI_GRADIENT) {
      kernels::face_scatter_kernel<C, NQ, double><<<unsigned((bi.num_face_nodes + 255) / 256), 256, 0, s>>>(
          f.ef64.p, bi.node_ptr.p, bi.node_ids.p, bi.node_ent.p, grad, bi.num_face_nodes, f.nnodes);
    }
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("face QoI launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

// adapts a QoI integrand to the per-element maker interface of the shape kernels
template <typename QF>
struct QoiMaker {
  QF qf;
  static constexpr int nparams = 0;
  SFX_HD QF operator()(const double*) const { return qf; }
};

template <int P, int C>
struct DomainQoiShapeFn {
  const sfx_form_s& f;
  const double* u;
  double t;
  cudaStream_t s;
  template <typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
    constexpr int EPW = 32 / NQ;
    if (f.ne == 0) return SFX_OK;
    kernels::DomainArgs<double> a{u, nullptr, nullptr, f.conn.p, nullptr, nullptr, nullptr, f.nnodes, f.ne, t};
    const int64_t warps = (f.ne + EPW - 1) / EPW;
    kernels::shape_adjoint_kernel<P, C, kernels::SHAPE_QOI, Nothing, QoiMaker<QF>>
        <<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(a, QoiMaker<QF>{qf}, f.Xe.p,
                                                            f.has_shape ? f.shape.p : nullptr, nullptr, f.eshape.p);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("QoI shape launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

template <int P, int C>
struct FaceQoiShapeFn {
  const sfx_form_s& f;
  const BoundaryIntegral& bi;
  const double* u;
  double* out;
  double t;
  cudaStream_t s;
  template <typename QF>
  int operator()(const QF& qf) {
    constexpr int NQ = (P + 1) * (P + 1);
    constexpr int FPW = 32 / NQ;
    if (bi.num_faces == 0) return SFX_OK;
    kernels::FaceArgs<double> a{u, nullptr, f.efshape.p, bi.fconn.p, bi.fgeom.p, f.nnodes, bi.num_faces, t};
    const int64_t warps = (bi.num_faces + FPW - 1) / FPW;
    kernels::face_shape_adjoint_kernel<P, C, kernels::SHAPE_QOI, QF><<<unsigned((warps * 32 + 127) / 128), 128, 0, s>>>(
        a, qf, bi.Xf.p, f.has_shape ? f.shape.p : nullptr, nullptr);
    kernels::face_scatter_kernel<3, NQ, double><<<unsigned((bi.num_face_nodes + 255) / 256), 256, 0, s>>>(
        f.efshape.p, bi.node_ptr.p, bi.node_ids.p, bi.node_ent.p, out, bi.num_face_nodes, f.nnodes);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("face QoI shape launch: ") + cudaGetErrorString(err));
    return SFX_OK;
  }
};

template <int P, int C>
int run_shape(sfx_form_s& f, double t, const double* u, double* out, cudaStream_t s) {
  if (int rc = ensure_shape_scratch(f)) return rc;
  SFX_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * size_t(3 * f.nnodes), s));
  for (const auto& qi : f.qoi_domain) {
    if (int rc = visit_domain_qoi<C>(qi, DomainQoiShapeFn<P, C>{f, u, t, s})) return rc;
    if (int rc = scatter_evector3(f, f.eshape.p, out, true, s)) return rc;
  }
  for (const auto& bi : f.qoi_boundary)
    if (int rc = visit_face_qoi<C>(bi, FaceQoiShapeFn<P, C>{f, bi, u, out, t, s})) return rc;
  return SFX_OK;
}

int check_qoi(sfx_form f) {
  if (!f) return fail(SFX_ERR_INVALID, "null form");
  if (!f->qoi) return fail(SFX_ERR_INVALID, "not a quantity of interest (create it with sfx_qoi_create)");
  return SFX_OK;
}

// number of per-element / per-face values of every integral of the QoI
int64_t value_count(const sfx_form_s& f) {
  int64_t n = f.ne * int64_t(f.qoi_domain.size());
  for (const auto& bi : f.qoi_boundary) n += bi.num_faces;
  return n;
}

// evaluates every integral in MODE into f.qoi_vals (and the gradient into
// grad), then sums the values into out[0]
template <int P, int C, int MODE>
int run(sfx_form_s& f, double t, const double* u, const double* du, double* grad, double* out, cudaStream_t s) {
  if constexpr (MODE == kernels::QOI_GRADIENT) SFX_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(double) * size_t(f.ndofs), s));
  const int64_t n = value_count(f);
  if (n == 0) {
    if (out) SFX_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double), s));
    return SFX_OK;
  }
  if (f.qoi_vals.n < size_t(n) && f.qoi_vals.alloc(size_t(n)) != cudaSuccess)
    return fail(SFX_ERR_NOMEM, "QoI value scratch");
  if (f.qoi_partial.n < size_t(kMaxQoiPartials) && f.qoi_partial.alloc(kMaxQoiPartials) != cudaSuccess)
    return fail(SFX_ERR_NOMEM, "QoI partial sums");
  int64_t at = 0;
  for (const auto& qi : f.qoi_domain) {
    if (int rc = visit_domain_qoi<C>(qi, DomainQoiFn<P, C, MODE>{f, u, du, f.qoi_vals.p + at, t, s})) return rc;
    if constexpr (MODE == kernels::QOI_GRADIENT)
      if (int rc = scatter_evector(f, f.e64.p, grad, true, s)) return rc;
    at += f.ne;
  }
  for (const auto& bi : f.qoi_boundary) {
    if (int rc = visit_face_qoi<C>(bi, FaceQoiFn<P, C, MODE>{f, bi, u, du, grad, f.qoi_vals.p + at, t, s})) return rc;
    at += bi.num_faces;
  }
  if (out) SFX_CUDA_TRY(kernels::qoi_sum(f.qoi_vals.p, n, f.qoi_partial.p, out, s));
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

template <int MODE>
int dispatch(sfx_form_s& f, double t, const double* u, const double* du, double* grad, double* out, cudaStream_t s) {
  if (f.qoi_domain.empty() && f.qoi_boundary.empty()) return fail(SFX_ERR_INVALID, "no integrals");
  if (f.p == 1 && f.c == 1) return run<1, 1, MODE>(f, t, u, du, grad, out, s);
  if (f.p == 1 && f.c == 3) return run<1, 3, MODE>(f, t, u, du, grad, out, s);
  if (f.p == 2 && f.c == 1) return run<2, 1, MODE>(f, t, u, du, grad, out, s);
  if (f.p == 2 && f.c == 3) return run<2, 3, MODE>(f, t, u, du, grad, out, s);
  return fail(SFX_ERR_UNSUPPORTED, "unsupported (order, components)");
}

}  // namespace

extern "C" {

int sfx_qoi_create(sfx_mesh mesh, int order, int components, sfx_form* out) {
  if (int rc = sfx_form_create(mesh, order, components, out)) return rc;
  (*out)->qoi = true;
  return SFX_OK;
}

int sfx_qoi_add_domain_integral(sfx_form qoi, int kind, const double* params) {
  if (int rc = check_qoi(qoi)) return rc;
  const int np = qoi_nparams(kind, qoi->c, false);
  if (np < 0) return fail(SFX_ERR_UNSUPPORTED, "QoI kind not available on the domain for this space");
  if (np > 0 && !params) return fail(SFX_ERR_INVALID, "QoI kind needs parameters");
  QoiIntegral qi;
  qi.kind = kind;
  if (np > 0) qi.params.assign(params, params + np);
  qoi->qoi_domain.push_back(std::move(qi));
  return SFX_OK;
}

int sfx_qoi_add_boundary_integral(sfx_form qoi, int kind, int side_mask, const double* params) {
  if (int rc = check_qoi(qoi)) return rc;
  const int np = qoi_nparams(kind, qoi->c, true);
  if (np < 0) return fail(SFX_ERR_UNSUPPORTED, "QoI kind not available on faces for this space");
  if (np > 0 && !params) return fail(SFX_ERR_INVALID, "QoI kind needs parameters");
  BoundaryIntegral bi;
  bi.material = kind;
  if (np > 0) bi.params.assign(params, params + np);
  if (int rc = build_faces(qoi, side_mask, bi)) return rc;
  qoi->qoi_boundary.push_back(std::move(bi));
  return SFX_OK;
}

int sfx_qoi_create_from_table(int order, int components, int64_t num_elements, int64_t num_nodes,
                              const int32_t* elem_nodes, const double* elem_vertices, sfx_form* out) {
  if (int rc = sfx_form_create_from_table(order, components, num_elements, num_nodes, elem_nodes, elem_vertices, out))
    return rc;
  (*out)->qoi = true;
  return SFX_OK;
}

int sfx_qoi_add_boundary_integral_faces(sfx_form qoi, int kind, int64_t num_faces, const int32_t* face_elem,
                                        const int32_t* face_side, const double* params) {
  if (int rc = check_qoi(qoi)) return rc;
  const int np = qoi_nparams(kind, qoi->c, true);
  if (np < 0) return fail(SFX_ERR_UNSUPPORTED, "QoI kind not available on faces for this space");
  if (np > 0 && !params) return fail(SFX_ERR_INVALID, "QoI kind needs parameters");
  BoundaryIntegral bi;
  bi.material = kind;
  if (np > 0) bi.params.assign(params, params + np);
  if (int rc = build_faces_list(qoi, num_faces, face_elem, face_side, bi)) return rc;
  qoi->qoi_boundary.push_back(std::move(bi));
  return SFX_OK;
}

int sfx_qoi_evaluate(sfx_form qoi, double t, const double* u, double* value, void* stream) {
  if (int rc = check_qoi(qoi)) return rc;
  if (!u || !value) return fail(SFX_ERR_INVALID, "null argument");
  return dispatch<kernels::QOI_VALUE>(*qoi, t, u, nullptr, nullptr, value, static_cast<cudaStream_t>(stream));
}

int sfx_qoi_gradient(sfx_form qoi, double t, const double* u, double* value, double* grad, void* stream) {
  if (int rc = check_qoi(qoi)) return rc;
  if (!u || !grad) return fail(SFX_ERR_INVALID, "null argument");
  return dispatch<kernels::QOI_GRADIENT>(*qoi, t, u, nullptr, grad, value, static_cast<cudaStream_t>(stream));
}

int sfx_qoi_shape_gradient(sfx_form qoi, double t, const double* u, double* out, void* stream) {
  if (int rc = check_qoi(qoi)) return rc;
  if (!u || !out) return fail(SFX_ERR_INVALID, "null argument");
  if (qoi->qoi_domain.empty() && qoi->qoi_boundary.empty()) return fail(SFX_ERR_INVALID, "no integrals");
  auto s = static_cast<cudaStream_t>(stream);
  sfx_form_s& f = *qoi;
  if (f.p == 1 && f.c == 1) return run_shape<1, 1>(f, t, u, out, s);
  if (f.p == 1 && f.c == 3) return run_shape<1, 3>(f, t, u, out, s);
  if (f.p == 2 && f.c == 1) return run_shape<2, 1>(f, t, u, out, s);
  if (f.p == 2 && f.c == 3) return run_shape<2, 3>(f, t, u, out, s);
  return fail(SFX_ERR_UNSUPPORTED, "unsupported (order, components)");
}

int sfx_qoi_action(sfx_form qoi, double t, const double* u, const double* du, double* out, void* stream) {
  if (int rc = check_qoi(qoi)) return rc;
  if (!u || !du || !out) return fail(SFX_ERR_INVALID, "null argument");
  return dispatch<kernels::QOI_ACTION>(*qoi, t, u, du, nullptr, out, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
