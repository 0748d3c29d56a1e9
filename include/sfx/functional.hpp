// sfx — serac::Functional's C++ interface for user q-functions (header-only;
// compile the including translation unit with nvcc, link libsfx_gb300.so).
//
//   sfx::Mesh mesh = sfx::Mesh::StructuredHex(nx, ny, nz, vertices);
//   sfx::Functional<sfx::H1<2, 3>(sfx::H1<2, 3>)> residual(mesh);
//   residual.AddDomainIntegral(sfx::Dimension<3>{}, sfx::DependsOn<0>{}, MyQFunction{...});
//   const double* r = residual(t, u);                          // device pointers
//   auto [r2, dRdu] = residual(t, sfx::differentiate_wrt(u));
//   dRdu.Mult(du, dr);                                         // FP64; MultF32 for the FP32 action
//   sfx::CSRMatrix K = sfx::assemble(dRdu);
//
// Mirrors functional.hpp:189-745 (Functional), :286-317 (AddDomainIntegral),
// :446-513 (operator()), :534-708 (Gradient, assemble), :523 (updateQdata)
// and quadrature_data.hpp:111-144 (QuadratureData).  The q-function is a
// callable object whose operator() is a template usable on the device
// (`SFX_HD`), called as qf(t, tuple{X, dX_dxi}, [state&,] tuple{u, du_dX}),
// the way serac's GPU-ready materials are functors (solid_mechanics.hpp:809-850).
// Its kernels are instantiated here, in the caller's translation unit, from
// sfx/kernels.cuh; mesh tables, geometric factors and the scatter-add come
// from the C ABI.
//
// Scope of this version: Functional<H1<p,c>(H1<p,c>)> with domain integrals
// over the whole mesh and boundary integrals over box sides or face lists;
// Functional<H1<p,3>(H1<p,c0>, H1<p,c1>, ...)> with domain integrals under
// DependsOn<i...> (several trial fields, derivatives and transposed actions
// with respect to any of them); quantities of interest; all with user
// q-functions (the C ABI material library serves callers without a compiler).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "sfx.h"
#include "sfx/boundary.cuh"
#include "sfx/kernels.cuh"
#include "sfx/multifield.cuh"
#include "sfx/qoi.cuh"
#include "sfx/sensitivity.cuh"

namespace sfx {

template <int p, int c = 1>
struct H1 {
  static constexpr int order = p;
  static constexpr int components = c;
};
template <int d>
struct Dimension {};
template <int... i>
struct DependsOn {};

struct differentiate_wrt_this {
  const double* u;
};
inline differentiate_wrt_this differentiate_wrt(const double* u) { return {u}; }

inline void check(int rc) {
  if (rc != SFX_OK) throw std::runtime_error(std::string("sfx: ") + sfx_last_error());
}
inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
struct DeviceArray {
  T* p = nullptr;
  size_t n = 0;
  DeviceArray() = default;
  explicit DeviceArray(size_t count) { resize(count); }
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  ~DeviceArray() {
    if (p) cudaFree(p);
  }
  void resize(size_t count) {
    if (count == n) return;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count) check_cuda(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
    n = count;
  }
};

class Mesh {
 public:
  static Mesh StructuredHex(int nx, int ny, int nz, const double* vertices) {
    Mesh m;
    sfx_mesh h = nullptr;
    check(sfx_mesh_create_structured_hex(nx, ny, nz, vertices, &h));
    m.h_ = std::shared_ptr<sfx_mesh_s>(h, [](sfx_mesh x) { sfx_mesh_destroy(x); });
    m.nx = nx;
    m.ny = ny;
    m.nz = nz;
    return m;
  }
  /// Any conforming hexahedral mesh as an element-node table of one order
  /// (host arrays: elem_nodes [ne][(order+1)^3] lexicographic, the caller's
  /// node numbering; elem_vertices [ne][8][3]), e.g. an mfem element-dof table;
  /// forms on it are built by sfx_form_create_from_table.
  static Mesh FromTable(int order, int64_t num_elements, int64_t num_nodes, const int32_t* elem_nodes,
                        const double* elem_vertices) {
    Mesh m;
    const int64_t npe = int64_t(order + 1) * (order + 1) * (order + 1);
    m.table_ = std::make_shared<Table>();
    m.table_->order = order;
    m.table_->num_elements = num_elements;
    m.table_->num_nodes = num_nodes;
    m.table_->nodes.assign(elem_nodes, elem_nodes + num_elements * npe);
    m.table_->vertices.assign(elem_vertices, elem_vertices + num_elements * 24);
    return m;
  }
  sfx_mesh handle() const { return h_.get(); }
  bool is_table() const { return table_ != nullptr; }
  /// a new form (or QoI) of order p with c components on this mesh
  sfx_form create(int p, int c, bool qoi) const {
    sfx_form h = nullptr;
    if (table_) {
      if (p != table_->order) throw std::runtime_error("sfx: the space order must be the element table's order");
      check(qoi ? sfx_qoi_create_from_table(p, c, table_->num_elements, table_->num_nodes, table_->nodes.data(),
                                            table_->vertices.data(), &h)
                : sfx_form_create_from_table(p, c, table_->num_elements, table_->num_nodes, table_->nodes.data(),
                                             table_->vertices.data(), &h));
    } else {
      check(qoi ? sfx_qoi_create(h_.get(), p, c, &h) : sfx_form_create(h_.get(), p, c, &h));
    }
    return h;
  }
  int nx = 0, ny = 0, nz = 0;

 private:
  struct Table {
    int order = 0;
    int64_t num_elements = 0, num_nodes = 0;
    std::vector<int32_t> nodes;
    std::vector<double> vertices;
  };
  std::shared_ptr<sfx_mesh_s> h_;
  std::shared_ptr<Table> table_;
};

/// Quadrature-point state (quadrature_data.hpp:111-144): one State per point,
/// stored on the device structure-of-arrays (doubles).
template <typename State>
class QuadratureData {
 public:
  QuadratureData(int64_t num_elements, int points_per_element, const State& init = State{})
      : num_points_(num_elements * points_per_element) {
    constexpr int k = int(sizeof(State) / sizeof(double));
    static_assert(sizeof(State) % sizeof(double) == 0, "state must be made of doubles");
    data_.resize(size_t(num_points_) * k);
    std::vector<double> host(size_t(num_points_) * k);
    const double* s = reinterpret_cast<const double*>(&init);
    for (int j = 0; j < k; j++)
      for (int64_t q = 0; q < num_points_; q++) host[size_t(j * num_points_ + q)] = s[j];
    check_cuda(cudaMemcpy(data_.p, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice), "qdata");
  }
  double* device() { return data_.p; }
  int64_t num_points() const { return num_points_; }
  State get(int64_t point) const {
    constexpr int k = int(sizeof(State) / sizeof(double));
    State out{};
    double* d = reinterpret_cast<double*>(&out);
    for (int j = 0; j < k; j++)
      check_cuda(cudaMemcpy(d + j, data_.p + j * num_points_ + point, sizeof(double), cudaMemcpyDeviceToHost), "qdata");
    return out;
  }

 private:
  int64_t num_points_;
  DeviceArray<double> data_;
};

struct CSRMatrix {
  int64_t rows = 0, nnz = 0;
  std::shared_ptr<DeviceArray<int64_t>> row_ptr;
  std::shared_ptr<DeviceArray<int32_t>> col;
  std::shared_ptr<DeviceArray<double>> values;
};

namespace detail {

// adapts a user q-function object to the kernels' per-element "maker" interface
template <typename QF>
struct UserMaker {
  QF qf;
  static constexpr int nparams = 0;
  static constexpr bool value_input = true;
  SFX_HD QF operator()(const double*) const { return qf; }
};

/// fn(graph) with the CSR column locator of the form behind the layout: the
/// analytic structured grid or the table form's scalar adjacency
template <typename Fn>
void with_graph(const sfx_form_layout& L, int p, Fn&& fn) {
  if (L.general) {
    fn(kernels::TableGraph{L.graph_ptr, L.graph_col, L.num_nodes});
    return;
  }
  kernels::GridShape g{};
  g.p = p;
  g.ne[0] = L.nx;
  g.ne[1] = L.ny;
  g.ne[2] = L.nz;
  for (int d = 0; d < 3; d++) g.N[d] = int64_t(p) * g.ne[d] + 1;
  fn(g);
}

/// out (+)= node-owner scatter of a 3-component E-vector [e][3][node] (shape space)
template <int NPE>
void scatter3(const sfx_form_layout& L, const double* E3, double* out, bool accumulate, cudaStream_t s) {
  if (L.num_nodes == 0) return;
  kernels::scatter_kernel<3, NPE, double><<<unsigned((L.num_nodes + 255) / 256), 256, 0, s>>>(
      E3, L.node_ptr, L.node_ent, out, L.num_nodes, accumulate, int64_t(0), L.num_nodes);
  check_cuda(cudaGetLastError(), "shape-space scatter");
}

inline unsigned warp_blocks(int64_t ne, int epw) {
  const int64_t warps = (ne + epw - 1) / epw;
  return unsigned((warps * 32 + 127) / 128);
}

struct IntegralBase {
  virtual ~IntegralBase() = default;
  virtual void residual(const sfx_form_layout& L, double t, const double* u, double* E, bool update,
                        cudaStream_t s) = 0;
  virtual void linearize(const sfx_form_layout& L, double t, const double* u, double* E, cudaStream_t s) = 0;
  virtual void jvp(const sfx_form_layout& L, const double* du, double* E, cudaStream_t s) = 0;
  virtual void jvp_f32(const sfx_form_layout& L, const float* du, float* E, cudaStream_t s) = 0;
  virtual void jvp_transpose(const sfx_form_layout& L, const double* v, double* E, cudaStream_t s) = 0;
  virtual void jvp_transpose_f32(const sfx_form_layout& L, const float* v, float* E, cudaStream_t s) = 0;
  virtual void diagonal(const sfx_form_layout& L, double* E, cudaStream_t s) = 0;
  virtual void element_matrices(const sfx_form_layout& L, double t, const double* u, double* K, int64_t e0,
                                int64_t e1, cudaStream_t s) = 0;
  // shape derivatives: dR_e/dp dshape into E [e][c][node]; (dR_e/dp)^T lam into E3 [e][3][node]
  virtual void shape_jvp(const sfx_form_layout& L, double t, const double* u, const double* dshape, double* E,
                         cudaStream_t s) = 0;
  virtual void shape_vjp(const sfx_form_layout& L, double t, const double* u, const double* lam, double* E3,
                         cudaStream_t s) = 0;
};

template <int P, int C, typename QF, typename State>
struct DomainIntegral : IntegralBase {
  using Maker = UserMaker<QF>;
  static constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
  static constexpr int EPW = 32 / NQ;
  static constexpr bool HS = kernels::tangent_has_source<C, State, QF>();
  using Shape = kernels::TangentShape<C, HS, true>;
  Maker maker;
  std::shared_ptr<QuadratureData<State>> qdata;
  DeviceArray<double> D64;
  DeviceArray<float> D32;

  DomainIntegral(const QF& qf, std::shared_ptr<QuadratureData<State>> q) : maker{qf}, qdata(std::move(q)) {}

  double* state_ptr() { return qdata ? qdata->device() : nullptr; }

  kernels::DomainArgs<double> args(const sfx_form_layout& L, double t, const double* u, const double* du, double* E) {
    return {u, du, E, L.conn, L.geom, state_ptr(), nullptr, L.num_nodes, L.num_elements, t};
  }
  void residual(const sfx_form_layout& L, double t, const double* u, double* E, bool update, cudaStream_t s) override {
    auto a = args(L, t, u, nullptr, E);
    if (update)
      kernels::domain_kernel<P, C, kernels::RESIDUAL_UPDATE, double, State, Maker>
          <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(a, maker);
    else
      kernels::domain_kernel<P, C, kernels::RESIDUAL, double, State, Maker>
          <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(a, maker);
    check_cuda(cudaGetLastError(), "residual kernel");
  }
  void linearize(const sfx_form_layout& L, double t, const double* u, double* E, cudaStream_t s) override {
    const size_t n = size_t(L.num_elements) * size_t(Shape::template stride<NQ>);
    D64.resize(n);
    D32.resize(n);
    auto a = args(L, t, u, nullptr, nullptr);
    kernels::linearize_kernel<P, C, State, Maker>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(a, maker, D64.p, D32.p, nullptr, E);
    check_cuda(cudaGetLastError(), "linearize kernel");
  }
  void jvp(const sfx_form_layout& L, const double* du, double* E, cudaStream_t s) override {
    kernels::jvp_stored_kernel<P, C, HS, true, double>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(du, D64.p, L.conn, E, L.num_nodes, L.num_elements);
    check_cuda(cudaGetLastError(), "jvp kernel");
  }
  void jvp_f32(const sfx_form_layout& L, const float* du, float* E, cudaStream_t s) override {
    kernels::jvp_stored_kernel<P, C, HS, true, float>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(du, D32.p, L.conn, E, L.num_nodes, L.num_elements);
    check_cuda(cudaGetLastError(), "jvp kernel (FP32)");
  }
  void jvp_transpose(const sfx_form_layout& L, const double* v, double* E, cudaStream_t s) override {
    kernels::jvp_stored_transpose_kernel<P, C, HS, true, double>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(v, D64.p, L.conn, E, L.num_nodes, L.num_elements);
    check_cuda(cudaGetLastError(), "transposed jvp kernel");
  }
  void jvp_transpose_f32(const sfx_form_layout& L, const float* v, float* E, cudaStream_t s) override {
    kernels::jvp_stored_transpose_kernel<P, C, HS, true, float>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(v, D32.p, L.conn, E, L.num_nodes, L.num_elements);
    check_cuda(cudaGetLastError(), "transposed jvp kernel (FP32)");
  }
  void diagonal(const sfx_form_layout& L, double* E, cudaStream_t s) override {
    kernels::diag_from_tangent_kernel<P, C, HS, true>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(D64.p, E, L.num_elements);
    check_cuda(cudaGetLastError(), "diagonal kernel");
  }
  void element_matrices(const sfx_form_layout& L, double t, const double* u, double* K, int64_t e0, int64_t e1,
                        cudaStream_t s) override {
    auto a = args(L, t, u, nullptr, K);
    kernels::element_matrix_kernel<P, C, State, Maker, false>
        <<<warp_blocks(e1 - e0, EPW), 128, 0, s>>>(a, maker, e0, e1);
    check_cuda(cudaGetLastError(), "element matrix kernel");
  }
  void shape_jvp(const sfx_form_layout& L, double t, const double* u, const double* dshape, double* E,
                 cudaStream_t s) override {
    auto a = args(L, t, u, nullptr, E);
    kernels::shape_jvp_kernel<P, C, State, Maker>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(a, maker, L.elem_vertices, L.shape, dshape);
    check_cuda(cudaGetLastError(), "shape jvp kernel");
  }
  void shape_vjp(const sfx_form_layout& L, double t, const double* u, const double* lam, double* E3,
                 cudaStream_t s) override {
    auto a = args(L, t, u, nullptr, nullptr);
    kernels::shape_adjoint_kernel<P, C, kernels::SHAPE_VJP, State, Maker>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(a, maker, L.elem_vertices, L.shape, lam, E3);
    check_cuda(cudaGetLastError(), "shape vjp kernel");
  }
};

template <typename T>
__global__ void to_f32_kernel(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) y[i] = float(x[i]);
}

/// A boundary integral of a user q-function over a face set
/// (AddBoundaryIntegral, functional.hpp:328-354): qf(t, tuple{X, dX/d(s,t)},
/// tuple{u, du/d(s,t)}) returns the flux per unit reference area (a scalar or
/// a c-vector), integrated with |dX/ds x dX/dt| over the faces.  Jacobian
/// actions re-evaluate the q-function on directional duals; the diagonal and
/// the CSR values come from face element matrices.  Every result is added to
/// its output through the face set's deterministic node-owner scatter.
template <int P, int C, typename QF>
struct BoundaryIntegral {
  static constexpr int NQ = (P + 1) * (P + 1);
  static constexpr int FPW = 32 / NQ;
  QF qf;
  int face_set = -1;
  sfx_face_layout F{};
  DeviceArray<double> E;
  DeviceArray<double> E3;  // shape-space face E-vector
  DeviceArray<float> E32;
  DeviceArray<double> K;

  unsigned blocks() const { return warp_blocks(F.num_faces, FPW); }
  unsigned scatter_blocks() const { return unsigned((F.num_face_nodes + 255) / 256); }
  template <typename Real>
  kernels::FaceArgs<Real> args(const sfx_form_layout& L, const Real* u, const Real* du, Real* out, double t) const {
    return {u, du, out, F.fconn, F.fgeom, L.num_nodes, F.num_faces, t};
  }
  // out += R_boundary(t, u)
  void residual(const sfx_form_layout& L, double t, const double* u, double* out, cudaStream_t s) {
    if (F.num_faces == 0) return;
    E.resize(size_t(F.num_faces) * C * NQ);
    kernels::face_kernel<P, C, kernels::RESIDUAL, double, QF><<<blocks(), 128, 0, s>>>(args(L, u, (const double*)nullptr, E.p, t), qf);
    kernels::face_scatter_kernel<C, NQ, double><<<scatter_blocks(), 256, 0, s>>>(
        E.p, F.node_ptr, F.node_ids, F.node_ent, out, F.num_face_nodes, L.num_nodes);
    check_cuda(cudaGetLastError(), "boundary residual kernel");
  }
  // out += dR_boundary/du(t, u) du (FP64 or FP32 throughout)
  template <typename Real>
  void jvp(const sfx_form_layout& L, double t, const Real* u, const Real* du, Real* out, cudaStream_t s) {
    if (F.num_faces == 0) return;
    Real* e;
    if constexpr (std::is_same<Real, double>::value) {
      E.resize(size_t(F.num_faces) * C * NQ);
      e = E.p;
    } else {
      E32.resize(size_t(F.num_faces) * C * NQ);
      e = E32.p;
    }
    kernels::face_kernel<P, C, kernels::JVP, Real, QF><<<blocks(), 128, 0, s>>>(args(L, u, du, e, t), qf);
    kernels::face_scatter_kernel<C, NQ, Real><<<scatter_blocks(), 256, 0, s>>>(
        e, F.node_ptr, F.node_ids, F.node_ent, out, F.num_face_nodes, L.num_nodes);
    check_cuda(cudaGetLastError(), "boundary jvp kernel");
  }
  // out += dR_boundary/du(t, u)^T v (FP64 or FP32 throughout)
  template <typename Real>
  void jvp_transpose(const sfx_form_layout& L, double t, const Real* u, const Real* v, Real* out, cudaStream_t s) {
    if (F.num_faces == 0) return;
    Real* e;
    if constexpr (std::is_same<Real, double>::value) {
      E.resize(size_t(F.num_faces) * C * NQ);
      e = E.p;
    } else {
      E32.resize(size_t(F.num_faces) * C * NQ);
      e = E32.p;
    }
    kernels::face_jvp_transpose_kernel<P, C, Real, QF><<<blocks(), 128, 0, s>>>(args(L, u, v, e, t), qf);
    kernels::face_scatter_kernel<C, NQ, Real><<<scatter_blocks(), 256, 0, s>>>(
        e, F.node_ptr, F.node_ids, F.node_ent, out, F.num_face_nodes, L.num_nodes);
    check_cuda(cudaGetLastError(), "boundary transposed jvp kernel");
  }
  // out += dR_boundary/dp (t, u) dshape
  void shape_jvp(const sfx_form_layout& L, double t, const double* u, const double* dshape, double* out,
                 cudaStream_t s) {
    if (F.num_faces == 0) return;
    E.resize(size_t(F.num_faces) * C * NQ);
    kernels::face_shape_jvp_kernel<P, C, QF><<<blocks(), 128, 0, s>>>(args(L, u, (const double*)nullptr, E.p, t), qf,
                                                                      F.face_vertices, L.shape, dshape);
    kernels::face_scatter_kernel<C, NQ, double><<<scatter_blocks(), 256, 0, s>>>(
        E.p, F.node_ptr, F.node_ids, F.node_ent, out, F.num_face_nodes, L.num_nodes);
    check_cuda(cudaGetLastError(), "boundary shape jvp kernel");
  }
  // out3 += (dR_boundary/dp (t, u))^T lam  (3 x num_nodes)
  void shape_vjp(const sfx_form_layout& L, double t, const double* u, const double* lam, double* out3,
                 cudaStream_t s) {
    if (F.num_faces == 0) return;
    E3.resize(size_t(F.num_faces) * 3 * NQ);
    kernels::face_shape_adjoint_kernel<P, C, kernels::SHAPE_VJP, QF><<<blocks(), 128, 0, s>>>(
        args(L, u, (const double*)nullptr, E3.p, t), qf, F.face_vertices, L.shape, lam);
    kernels::face_scatter_kernel<3, NQ, double><<<scatter_blocks(), 256, 0, s>>>(
        E3.p, F.node_ptr, F.node_ids, F.node_ent, out3, F.num_face_nodes, L.num_nodes);
    check_cuda(cudaGetLastError(), "boundary shape vjp kernel");
  }
  // face element matrices at (t, u), then += into the diagonal and / or the CSR values
  void matrices(const sfx_form_layout& L, double t, const double* u, double* diag, double* values, cudaStream_t s) {
    if (F.num_faces == 0) return;
    K.resize(size_t(F.num_faces) * (C * NQ) * (C * NQ));
    kernels::face_matrix_kernel<P, C, QF><<<blocks(), 128, 0, s>>>(args(L, u, (const double*)nullptr, K.p, t), qf);
    if (diag)
      kernels::face_diag_kernel<C, NQ><<<scatter_blocks(), 256, 0, s>>>(F.node_ptr, F.node_ids, F.node_ent, K.p, diag,
                                                                         F.num_face_nodes, L.num_nodes);
    if (values) {
      with_graph(L, P, [&](auto g) {
        kernels::face_csr_kernel<P, C><<<unsigned((F.num_face_nodes * C + 127) / 128), 128, 0, s>>>(
            g, L.row_ptr, F.fconn, F.node_ptr, F.node_ids, F.node_ent, K.p, values, F.num_face_nodes);
      });
    }
    check_cuda(cudaGetLastError(), "boundary matrix kernels");
  }
};

struct BoundaryBase {
  virtual ~BoundaryBase() = default;
  virtual void residual(const sfx_form_layout& L, double t, const double* u, double* out, cudaStream_t s) = 0;
  virtual void jvp(const sfx_form_layout& L, double t, const double* u, const double* du, double* out,
                   cudaStream_t s) = 0;
  virtual void jvp_f32(const sfx_form_layout& L, double t, const float* u, const float* du, float* out,
                       cudaStream_t s) = 0;
  virtual void jvp_transpose(const sfx_form_layout& L, double t, const double* u, const double* v, double* out,
                             cudaStream_t s) = 0;
  virtual void shape_jvp(const sfx_form_layout& L, double t, const double* u, const double* dshape, double* out,
                         cudaStream_t s) = 0;
  virtual void shape_vjp(const sfx_form_layout& L, double t, const double* u, const double* lam, double* out3,
                         cudaStream_t s) = 0;
  virtual void jvp_transpose_f32(const sfx_form_layout& L, double t, const float* u, const float* v, float* out,
                                 cudaStream_t s) = 0;
  virtual void matrices(const sfx_form_layout& L, double t, const double* u, double* diag, double* values,
                        cudaStream_t s) = 0;
};
template <int P, int C, typename QF>
struct BoundaryHolder : BoundaryBase {
  BoundaryIntegral<P, C, QF> b;
  void residual(const sfx_form_layout& L, double t, const double* u, double* out, cudaStream_t s) override {
    b.residual(L, t, u, out, s);
  }
  void jvp(const sfx_form_layout& L, double t, const double* u, const double* du, double* out,
           cudaStream_t s) override {
    b.template jvp<double>(L, t, u, du, out, s);
  }
  void jvp_f32(const sfx_form_layout& L, double t, const float* u, const float* du, float* out,
               cudaStream_t s) override {
    b.template jvp<float>(L, t, u, du, out, s);
  }
  void jvp_transpose(const sfx_form_layout& L, double t, const double* u, const double* v, double* out,
                     cudaStream_t s) override {
    b.template jvp_transpose<double>(L, t, u, v, out, s);
  }
  void shape_jvp(const sfx_form_layout& L, double t, const double* u, const double* dshape, double* out,
                 cudaStream_t s) override {
    b.shape_jvp(L, t, u, dshape, out, s);
  }
  void shape_vjp(const sfx_form_layout& L, double t, const double* u, const double* lam, double* out3,
                 cudaStream_t s) override {
    b.shape_vjp(L, t, u, lam, out3, s);
  }
  void jvp_transpose_f32(const sfx_form_layout& L, double t, const float* u, const float* v, float* out,
                         cudaStream_t s) override {
    b.template jvp_transpose<float>(L, t, u, v, out, s);
  }
  void matrices(const sfx_form_layout& L, double t, const double* u, double* diag, double* values,
                cudaStream_t s) override {
    b.matrices(L, t, u, diag, values, s);
  }
};

}  // namespace detail

template <typename Signature>
class Functional;

/// Functional<H1<p,c>(H1<p,c>)>: residual, linearisation and assembly of the
/// domain integrals added to it.  Vectors are device pointers (byNODES).
template <int p, int c>
class Functional<H1<p, c>(H1<p, c>)> {
 public:
  class Gradient {
   public:
    explicit Gradient(Functional* f) : f_(f) {}
    /// df = dR/du(t_lin, u_lin) dx  (functional.hpp:556-559)
    void Mult(const double* dx, double* df, cudaStream_t s = nullptr) const { f_->jvp(dx, df, s); }
    /// FP32 action on the FP32 copy of the stored tangent
    void MultF32(const float* dx, float* df, cudaStream_t s = nullptr) const { f_->jvp_f32(dx, df, s); }
    /// df = dR/du^T v (mfem::Operator::MultTranspose), the adjoint action, from
    /// the stored tangent transposed; FP32 on the FP32 copy
    void MultTranspose(const double* v, double* df, cudaStream_t s = nullptr) const { f_->jvp_transpose(v, df, s); }
    void MultTransposeF32(const float* v, float* df, cudaStream_t s = nullptr) const {
      f_->jvp_transpose_f32(v, df, s);
    }
    /// returns a member buffer overwritten by the next call (functional.hpp:562-566)
    const double* operator()(const double* dx) {
      Mult(dx, f_->df_.p);
      return f_->df_.p;
    }
    void AssembleDiagonal(double* diag, cudaStream_t s = nullptr) const { f_->diagonal(diag, s); }
    friend CSRMatrix assemble(Gradient& g) { return g.f_->assemble_csr(); }

   private:
    Functional* f_;
  };

  explicit Functional(const Mesh& mesh) : mesh_(mesh), grad_(this) {
    sfx_form h = mesh.create(p, c, false);
    form_ = std::shared_ptr<sfx_form_s>(h, [](sfx_form x) { sfx_form_destroy(x); });
    check(sfx_form_get_layout(h, &L_));
    out_.resize(size_t(L_.num_dofs));
    df_.resize(size_t(L_.num_dofs));
    u_lin_.resize(size_t(L_.num_dofs));
  }

  static constexpr int points_per_element = (p + 1) * (p + 1) * (p + 1);
  int64_t num_dofs() const { return L_.num_dofs; }
  int64_t num_elements() const { return L_.num_elements; }

  /// AddDomainIntegral(Dimension<3>, DependsOn<0>, qf[, qdata])  (functional.hpp:286-317).
  /// A q-function that takes a state argument but gets no quadrature data
  /// receives an Empty state (serac's EmptyQData).
  template <typename QF>
  void AddDomainIntegral(Dimension<3>, DependsOn<0>, const QF& qf) {
    using Pos = tuple<tensor<double, 3>, tensor<double, 3, 3>>;
    using Arg = tuple<kernels::value_t<c, double>, kernels::grad_t<c, double>>;
    if constexpr (std::is_invocable<const QF&, double, Pos, Arg>::value) {
      integrals_.emplace_back(new detail::DomainIntegral<p, c, QF, Nothing>(qf, nullptr));
    } else {
      integrals_.emplace_back(new detail::DomainIntegral<p, c, QF, Empty>(qf, nullptr));
    }
  }
  template <typename QF, typename State>
  void AddDomainIntegral(Dimension<3>, DependsOn<0>, const QF& qf, std::shared_ptr<QuadratureData<State>> qdata) {
    integrals_.emplace_back(new detail::DomainIntegral<p, c, QF, State>(qf, std::move(qdata)));
  }
  template <typename QF>
  void AddVolumeIntegral(DependsOn<0> d, const QF& qf) {
    AddDomainIntegral(Dimension<3>{}, d, qf);
  }

  /// AddBoundaryIntegral(Dimension<2>, DependsOn<0>, qf, sides) (functional.hpp:328-354)
  /// over the faces of the box sides in side_mask (bit s-1 for side s: 1 z=0,
  /// 2 y=0, 3 x=1, 4 y=1, 5 x=0, 6 z=1); qf(t, tuple{X, dX/d(s,t)},
  /// tuple{u, du/d(s,t)}) returns the boundary flux (scalar or c-vector).
  template <typename QF>
  void AddBoundaryIntegral(Dimension<2>, DependsOn<0>, const QF& qf, int side_mask) {
    auto h = std::make_unique<detail::BoundaryHolder<p, c, QF>>();
    h->b.qf = qf;
    check(sfx_form_add_face_set(form_.get(), side_mask, &h->b.face_set));
    check(sfx_form_get_face_layout(form_.get(), h->b.face_set, &h->b.F));
    boundary_.push_back(std::move(h));
  }
  template <typename QF>
  void AddSurfaceIntegral(DependsOn<0> d, const QF& qf, int side_mask) {
    AddBoundaryIntegral(Dimension<2>{}, d, qf, side_mask);
  }
  /// the same over a face list: face_elem[k] an element, face_side[k] its
  /// local side (1..6, the box-side numbering in the element's own frame)
  template <typename QF>
  void AddBoundaryIntegral(Dimension<2>, DependsOn<0>, const QF& qf, const std::vector<int32_t>& face_elem,
                           const std::vector<int32_t>& face_side) {
    if (face_elem.size() != face_side.size()) throw std::runtime_error("sfx: face lists differ in length");
    auto h = std::make_unique<detail::BoundaryHolder<p, c, QF>>();
    h->b.qf = qf;
    check(sfx_form_add_face_set_faces(form_.get(), int64_t(face_elem.size()), face_elem.data(), face_side.data(),
                                      &h->b.face_set));
    check(sfx_form_get_face_layout(form_.get(), h->b.face_set, &h->b.F));
    boundary_.push_back(std::move(h));
  }

  /// updateQdata(bool) (functional.hpp:523): commit quadrature state on residual calls
  void updateQdata(bool flag) { update_qdata_ = flag; }

  /// Shape displacement p (device, 3 * num_nodes doubles, byNODES; nullptr =
  /// none): the integrals are evaluated on X + p as ShapeAwareFunctional does
  /// (shape_aware_functional.hpp:45-172).  Linearise again afterwards.
  void SetShapeDisplacement(const double* shape, cudaStream_t s = nullptr) {
    check(sfx_form_set_shape_displacement(form_.get(), shape, s));
    check(sfx_form_get_layout(form_.get(), &L_));  // the shape field's device address
    linearized_ = false;
  }

  /// dr = dR/dp (t, u; p) dshape: the residual differentiated with respect to
  /// the shape displacement set on the form (ShapeAwareFunctional's argument 0,
  /// shape_aware_functional.hpp:537-541); dshape: device, 3 * num_nodes doubles
  void ShapeJvp(double t, const double* u, const double* dshape, double* dr, cudaStream_t s = nullptr) {
    if (integrals_.empty() && boundary_.empty()) throw std::runtime_error("sfx: no integrals");
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(dr, 0, sizeof(double) * size_t(L_.num_dofs), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->shape_jvp(L_, t, u, dshape, L_.evector, s);
      check(sfx_scatter_add(form_.get(), L_.evector, dr, i > 0, s));
    }
    for (auto& b : boundary_) b->shape_jvp(L_, t, u, dshape, dr, s);
  }
  /// out = (dR/dp (t, u; p))^T lam (3 * num_nodes): the adjoint shape
  /// sensitivity (computeTimestepShapeSensitivity, solid_mechanics.hpp:1421-1431)
  void ShapeVjp(double t, const double* u, const double* lam, double* out, cudaStream_t s = nullptr) {
    if (integrals_.empty() && boundary_.empty()) throw std::runtime_error("sfx: no integrals");
    e3_.resize(size_t(L_.num_elements) * points_per_element * 3);
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(out, 0, sizeof(double) * size_t(3 * L_.num_nodes), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->shape_vjp(L_, t, u, lam, e3_.p, s);
      detail::scatter3<points_per_element>(L_, e3_.p, out, i > 0, s);
    }
    for (auto& b : boundary_) b->shape_vjp(L_, t, u, lam, out, s);
  }

  /// R(t, u) into a member buffer (functional.hpp:502-513)
  const double* operator()(double t, const double* u, cudaStream_t s = nullptr) {
    residual(t, u, out_.p, s);
    return out_.p;
  }
  void residual(double t, const double* u, double* r, cudaStream_t s = nullptr) {
    if (integrals_.empty() && boundary_.empty()) throw std::runtime_error("sfx: no integrals");
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(r, 0, sizeof(double) * size_t(L_.num_dofs), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->residual(L_, t, u, L_.evector, update_qdata_, s);
      check(sfx_scatter_add(form_.get(), L_.evector, r, i > 0, s));
    }
    for (auto& b : boundary_) b->residual(L_, t, u, r, s);
  }

  /// (R(t, u), dR/du) with the tangent linearised at u (functional.hpp:481-489)
  std::tuple<const double*, Gradient&> operator()(double t, differentiate_wrt_this w, cudaStream_t s = nullptr) {
    if (integrals_.empty() && boundary_.empty()) throw std::runtime_error("sfx: no integrals");
    check_cuda(cudaMemcpyAsync(u_lin_.p, w.u, sizeof(double) * size_t(L_.num_dofs), cudaMemcpyDeviceToDevice, s),
               "copy u");
    t_lin_ = t;
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(out_.p, 0, sizeof(double) * size_t(L_.num_dofs), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->linearize(L_, t, u_lin_.p, L_.evector, s);
      check(sfx_scatter_add(form_.get(), L_.evector, out_.p, i > 0, s));
    }
    if (!boundary_.empty()) {
      u_lin32_.resize(size_t(L_.num_dofs));
      detail::to_f32_kernel<float><<<unsigned((L_.num_dofs + 255) / 256), 256, 0, s>>>(u_lin_.p, u_lin32_.p,
                                                                                       L_.num_dofs);
      for (auto& b : boundary_) b->residual(L_, t, u_lin_.p, out_.p, s);
    }
    linearized_ = true;
    return {out_.p, grad_};
  }

 private:
  friend class Gradient;
  void require_linearized() const {
    if (!linearized_) throw std::runtime_error("sfx: linearise with operator()(t, differentiate_wrt(u)) first");
  }
  void jvp(const double* dx, double* df, cudaStream_t s) {
    require_linearized();
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(df, 0, sizeof(double) * size_t(L_.num_dofs), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->jvp(L_, dx, L_.evector, s);
      check(sfx_scatter_add(form_.get(), L_.evector, df, i > 0, s));
    }
    for (auto& b : boundary_) b->jvp(L_, t_lin_, u_lin_.p, dx, df, s);
  }
  void jvp_f32(const float* dx, float* df, cudaStream_t s) {
    require_linearized();
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(df, 0, sizeof(float) * size_t(L_.num_dofs), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->jvp_f32(L_, dx, L_.evector_f32, s);
      check(sfx_scatter_add_f32(form_.get(), L_.evector_f32, df, i > 0, s));
    }
    for (auto& b : boundary_) b->jvp_f32(L_, t_lin_, u_lin32_.p, dx, df, s);
  }
  void jvp_transpose(const double* v, double* df, cudaStream_t s) {
    require_linearized();
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(df, 0, sizeof(double) * size_t(L_.num_dofs), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->jvp_transpose(L_, v, L_.evector, s);
      check(sfx_scatter_add(form_.get(), L_.evector, df, i > 0, s));
    }
    for (auto& b : boundary_) b->jvp_transpose(L_, t_lin_, u_lin_.p, v, df, s);
  }
  void jvp_transpose_f32(const float* v, float* df, cudaStream_t s) {
    require_linearized();
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(df, 0, sizeof(float) * size_t(L_.num_dofs), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->jvp_transpose_f32(L_, v, L_.evector_f32, s);
      check(sfx_scatter_add_f32(form_.get(), L_.evector_f32, df, i > 0, s));
    }
    for (auto& b : boundary_) b->jvp_transpose_f32(L_, t_lin_, u_lin32_.p, v, df, s);
  }
  void diagonal(double* diag, cudaStream_t s) {
    require_linearized();
    if (integrals_.empty()) check_cuda(cudaMemsetAsync(diag, 0, sizeof(double) * size_t(L_.num_dofs), s), "memset");
    for (size_t i = 0; i < integrals_.size(); i++) {
      integrals_[i]->diagonal(L_, L_.evector, s);
      check(sfx_scatter_add(form_.get(), L_.evector, diag, i > 0, s));
    }
    for (auto& b : boundary_) b->matrices(L_, t_lin_, u_lin_.p, diag, nullptr, s);
  }

 public:
  /// assemble(Gradient&) (functional.hpp:569-667): CSR on the device
  CSRMatrix assemble_csr() {
    require_linearized();
    int64_t nnz = 0;
    check(sfx_csr_nnz(form_.get(), &nnz));
    check(sfx_form_get_layout(form_.get(), &L_));
    CSRMatrix A;
    A.rows = L_.num_dofs;
    A.nnz = nnz;
    A.row_ptr = std::make_shared<DeviceArray<int64_t>>(size_t(L_.num_dofs + 1));
    A.col = std::make_shared<DeviceArray<int32_t>>(size_t(nnz));
    A.values = std::make_shared<DeviceArray<double>>(size_t(nnz));
    check(sfx_csr_graph(form_.get(), A.row_ptr->p, A.col->p, nullptr));
    constexpr int NDOF = c * points_per_element;
    const int64_t chunk = std::min<int64_t>(L_.num_elements, 16384);
    DeviceArray<double> K(size_t(chunk) * NDOF * NDOF);
    bool first = true;
    for (auto& in : integrals_) {
      for (int64_t e0 = 0; e0 < L_.num_elements; e0 += chunk) {
        const int64_t e1 = std::min(L_.num_elements, e0 + chunk);
        in->element_matrices(L_, t_lin_, u_lin_.p, K.p, e0, e1, nullptr);
        detail::with_graph(L_, p, [&](auto g) {
          kernels::csr_assemble_kernel<p, c><<<unsigned((L_.num_dofs + 127) / 128), 128>>>(
              g, L_.row_ptr, L_.conn, L_.node_ptr, L_.node_ent, K.p, e0, e1, A.values->p, !first);
        });
        check_cuda(cudaGetLastError(), "assembly kernel");
        first = false;
      }
    }
    if (first) check_cuda(cudaMemsetAsync(A.values->p, 0, sizeof(double) * size_t(nnz), nullptr), "memset");
    for (auto& b : boundary_) b->matrices(L_, t_lin_, u_lin_.p, nullptr, A.values->p, nullptr);
    check_cuda(cudaDeviceSynchronize(), "assembly");
    return A;
  }

 private:
  Mesh mesh_;
  std::shared_ptr<sfx_form_s> form_;
  sfx_form_layout L_{};
  std::vector<std::unique_ptr<detail::IntegralBase>> integrals_;
  std::vector<std::unique_ptr<detail::BoundaryBase>> boundary_;
  DeviceArray<double> out_, df_, u_lin_, e3_;
  DeviceArray<float> u_lin32_;
  double t_lin_ = 0.0;
  bool linearized_ = false;
  bool update_qdata_ = false;
  Gradient grad_;
};

namespace detail {

// one integral of a quantity of interest: per-element / per-face values and,
// for QOI_GRADIENT, dQ/du added into grad
struct QoiBase {
  virtual ~QoiBase() = default;
  virtual int64_t count(const sfx_form_layout& L) const = 0;
  virtual void run(int mode, const sfx_form_layout& L, sfx_form form, double t, const double* u, const double* du,
                   double* vals, double* grad, cudaStream_t s) = 0;
  // out3 += dQ/dp (3 x num_nodes), E3: element scratch [e][3][node]
  virtual void shape_gradient(const sfx_form_layout& L, double t, const double* u, double* E3, double* out3,
                              cudaStream_t s) = 0;
};

template <int P, int C, typename QF>
struct QoiDomain : QoiBase {
  static constexpr int EPW = 32 / ((P + 1) * (P + 1) * (P + 1));
  QF qf;
  explicit QoiDomain(const QF& q) : qf(q) {}
  int64_t count(const sfx_form_layout& L) const override { return L.num_elements; }
  template <int MODE>
  void launch(const sfx_form_layout& L, double t, const double* u, const double* du, double* vals, cudaStream_t s) {
    kernels::DomainArgs<double> a{u, du, L.evector, L.conn, L.geom, nullptr, nullptr, L.num_nodes, L.num_elements, t};
    kernels::qoi_domain_kernel<P, C, MODE, QF><<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(a, qf, vals);
    check_cuda(cudaGetLastError(), "QoI kernel");
  }
  void shape_gradient(const sfx_form_layout& L, double t, const double* u, double* E3, double* out3,
                      cudaStream_t s) override {
    if (L.num_elements == 0) return;
    kernels::DomainArgs<double> a{u, nullptr, nullptr, L.conn, L.geom, nullptr, nullptr, L.num_nodes, L.num_elements, t};
    kernels::shape_adjoint_kernel<P, C, kernels::SHAPE_QOI, Nothing, UserMaker<QF>>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(a, UserMaker<QF>{qf}, L.elem_vertices, L.shape, nullptr, E3);
    check_cuda(cudaGetLastError(), "QoI shape kernel");
    scatter3<(P + 1) * (P + 1) * (P + 1)>(L, E3, out3, true, s);
  }
  void run(int mode, const sfx_form_layout& L, sfx_form form, double t, const double* u, const double* du,
           double* vals, double* grad, cudaStream_t s) override {
    if (L.num_elements == 0) return;
    if (mode == kernels::QOI_VALUE) launch<kernels::QOI_VALUE>(L, t, u, du, vals, s);
    if (mode == kernels::QOI_ACTION) launch<kernels::QOI_ACTION>(L, t, u, du, vals, s);
    if (mode == kernels::QOI_GRADIENT) {
      launch<kernels::QOI_GRADIENT>(L, t, u, du, vals, s);
      check(sfx_scatter_add(form, L.evector, grad, 1, s));
    }
  }
};

template <int P, int C, typename QF>
struct QoiFaces : QoiBase {
  static constexpr int NQ = (P + 1) * (P + 1);
  static constexpr int FPW = 32 / NQ;
  QF qf;
  int face_set = -1;
  sfx_face_layout F{};
  DeviceArray<double> E;
  DeviceArray<double> E3;
  explicit QoiFaces(const QF& q) : qf(q) {}
  int64_t count(const sfx_form_layout&) const override { return F.num_faces; }
  template <int MODE>
  void launch(const sfx_form_layout& L, double t, const double* u, const double* du, double* vals, cudaStream_t s) {
    kernels::FaceArgs<double> a{u, du, E.p, F.fconn, F.fgeom, L.num_nodes, F.num_faces, t};
    kernels::qoi_face_kernel<P, C, MODE, QF><<<warp_blocks(F.num_faces, FPW), 128, 0, s>>>(a, qf, vals);
    check_cuda(cudaGetLastError(), "face QoI kernel");
  }
  void shape_gradient(const sfx_form_layout& L, double t, const double* u, double*, double* out3,
                      cudaStream_t s) override {
    if (F.num_faces == 0) return;
    E3.resize(size_t(F.num_faces) * 3 * NQ);
    kernels::FaceArgs<double> a{u, nullptr, E3.p, F.fconn, F.fgeom, L.num_nodes, F.num_faces, t};
    kernels::face_shape_adjoint_kernel<P, C, kernels::SHAPE_QOI, QF><<<warp_blocks(F.num_faces, FPW), 128, 0, s>>>(
        a, qf, F.face_vertices, L.shape, nullptr);
    kernels::face_scatter_kernel<3, NQ, double><<<unsigned((F.num_face_nodes + 255) / 256), 256, 0, s>>>(
        E3.p, F.node_ptr, F.node_ids, F.node_ent, out3, F.num_face_nodes, L.num_nodes);
    check_cuda(cudaGetLastError(), "face QoI shape kernels");
  }
  void run(int mode, const sfx_form_layout& L, sfx_form, double t, const double* u, const double* du, double* vals,
           double* grad, cudaStream_t s) override {
    if (F.num_faces == 0) return;
    E.resize(size_t(F.num_faces) * C * NQ);
    if (mode == kernels::QOI_VALUE) launch<kernels::QOI_VALUE>(L, t, u, du, vals, s);
    if (mode == kernels::QOI_ACTION) launch<kernels::QOI_ACTION>(L, t, u, du, vals, s);
    if (mode == kernels::QOI_GRADIENT) {
      launch<kernels::QOI_GRADIENT>(L, t, u, du, vals, s);
      kernels::face_scatter_kernel<C, NQ, double><<<unsigned((F.num_face_nodes + 255) / 256), 256, 0, s>>>(
          E.p, F.node_ptr, F.node_ids, F.node_ent, grad, F.num_face_nodes, L.num_nodes);
      check_cuda(cudaGetLastError(), "face QoI scatter");
    }
  }
};

}  // namespace detail

namespace detail {

/// out (+)= node-owner scatter of a C-component E-vector [e][C][node]
template <int C, int NPE>
void scatter_c(const sfx_form_layout& L, const double* E, double* out, bool accumulate, cudaStream_t s) {
  if (L.num_nodes == 0) return;
  kernels::scatter_kernel<C, NPE, double><<<unsigned((L.num_nodes + 255) / 256), 256, 0, s>>>(
      E, L.node_ptr, L.node_ent, out, L.num_nodes, accumulate, int64_t(0), L.num_nodes);
  check_cuda(cudaGetLastError(), "multi-field scatter");
}

/// one multi-field domain integral (type-erased over the q-function and its
/// DependsOn arguments)
struct MultiIntegralBase {
  virtual ~MultiIntegralBase() = default;
  virtual void residual(const sfx_form_layout& L, double t, const double* const* fields, double* E,
                        cudaStream_t s) = 0;
  /// stores the derivative with respect to form field `field`; false if the integral does not read it
  virtual bool linearize(const sfx_form_layout& L, double t, const double* const* fields, int field,
                         cudaStream_t s) = 0;
  virtual void jvp(const sfx_form_layout& L, const double* d, double* E, cudaStream_t s) = 0;
  virtual void jvp_transpose(const sfx_form_layout& L, const double* v, double* E, cudaStream_t s) = 0;
};

template <int P, int CT, typename QF, typename State, typename Comps, int... I>
struct MultiIntegral;

template <int P, int CT, typename QF, typename State, int... C, int... I>
struct MultiIntegral<P, CT, QF, State, std::integer_sequence<int, C...>, I...> : MultiIntegralBase {
  static constexpr int NQ = (P + 1) * (P + 1) * (P + 1);
  static constexpr int EPW = 32 / NQ;
  static constexpr int form_comps[] = {C...};
  using FL = kernels::FieldList<form_comps[I]...>;
  static constexpr int args[] = {I...};
  struct Maker {
    QF qf;
    static constexpr int nparams = 0;
    SFX_HD QF operator()(const double*) const { return qf; }
  };
  Maker maker;
  DeviceArray<double> D;
  int W = -1;  // argument of the stored derivative

  explicit MultiIntegral(const QF& qf) : maker{qf} {}

  kernels::MultiArgs<double> margs(const sfx_form_layout& L, double t, const double* const* fields, const double* dir,
                                   double* E) const {
    kernels::MultiArgs<double> a{};
    for (int k = 0; k < int(sizeof...(I)); k++) a.u[k] = fields ? fields[args[k]] : nullptr;
    a.dir = dir;
    a.out_e = E;
    a.conn = L.conn;
    a.geom = L.geom;
    a.num_nodes = L.num_nodes;
    a.num_elements = L.num_elements;
    a.t = t;
    return a;
  }
  template <int w>
  void launch(const sfx_form_layout& L, double t, const double* const* fields, double* E, cudaStream_t s) {
    if constexpr (w >= 0) {
      constexpr int CW = FL::template comps<w>();
      D.resize(size_t(L.num_elements) * size_t(kernels::MultiTangentShape<CT, CW>::template stride<NQ>));
    }
    kernels::multi_domain_kernel<P, CT, FL, w, State, Maker>
        <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(margs(L, t, fields, nullptr, E), maker, D.p);
    check_cuda(cudaGetLastError(), "multi-field kernel");
  }
  void residual(const sfx_form_layout& L, double t, const double* const* fields, double* E, cudaStream_t s) override {
    launch<-1>(L, t, fields, E, s);
  }
  bool linearize(const sfx_form_layout& L, double t, const double* const* fields, int field, cudaStream_t s) override {
    W = -1;
    for (int k = 0; k < int(sizeof...(I)); k++)
      if (args[k] == field) W = k;
    switch (W) {
      case 0: launch<0>(L, t, fields, nullptr, s); break;
      case 1: if constexpr (sizeof...(I) > 1) launch<1>(L, t, fields, nullptr, s); break;
      case 2: if constexpr (sizeof...(I) > 2) launch<2>(L, t, fields, nullptr, s); break;
      case 3: if constexpr (sizeof...(I) > 3) launch<3>(L, t, fields, nullptr, s); break;
      default: return false;
    }
    return true;
  }
  template <bool TRANSPOSE>
  void action(const sfx_form_layout& L, const double* dir, double* E, cudaStream_t s) {
    auto run = [&](auto cw) {
      constexpr int CW = decltype(cw)::value;
      kernels::multi_jvp_kernel<P, CT, CW, TRANSPOSE>
          <<<warp_blocks(L.num_elements, EPW), 128, 0, s>>>(margs(L, 0.0, nullptr, dir, E), D.p);
    };
    const int cw = comps_of(W);
    if (cw == 1) run(std::integral_constant<int, 1>{});
    else if (cw == 3) run(std::integral_constant<int, 3>{});
    else throw std::runtime_error("sfx: field components must be 1 or 3");
    check_cuda(cudaGetLastError(), "multi-field action");
  }
  static int comps_of(int w) {
    constexpr int a[] = {form_comps[I]...};
    return (w >= 0 && w < int(sizeof...(I))) ? a[w] : 0;
  }
  void jvp(const sfx_form_layout& L, const double* d, double* E, cudaStream_t s) override { action<false>(L, d, E, s); }
  void jvp_transpose(const sfx_form_layout& L, const double* v, double* E, cudaStream_t s) override {
    action<true>(L, v, E, s);
  }
};

}  // namespace detail

/// Functional<H1<p,c>(H1<p,c0>, H1<p,c1>, ...)> (functional.hpp:189-317): a
/// residual of several trial fields, each H1 of the test space's order on the
/// same node grid, as SolidMechanics builds test(displacement, acceleration,
/// parameters...) (solid_mechanics.hpp:243).  AddDomainIntegral(Dimension<3>,
/// DependsOn<i...>, qf) passes the fields i... to qf(t, tuple{X, dX/dxi},
/// tuple{value, gradient}...) in that order; operator()(t, fields...) with one
/// field wrapped in differentiate_wrt returns (R, dR/d(that field)).
template <int p, int c, int c0, int c1, int... cs>
class Functional<H1<p, c>(H1<p, c0>, H1<p, c1>, H1<p, cs>...)> {
  static constexpr int nfields = 2 + int(sizeof...(cs));
  using Comps = std::integer_sequence<int, c0, c1, cs...>;
  static constexpr int comps_[] = {c0, c1, cs...};
  static constexpr int NPE = (p + 1) * (p + 1) * (p + 1);

 public:
  /// dR/d(field wrt) at the linearisation point
  class Gradient {
   public:
    explicit Gradient(Functional* f) : f_(f) {}
    /// df = dR/d(field) d (test space)
    void Mult(const double* d, double* df, cudaStream_t s = nullptr) const { f_->jvp(d, df, s); }
    /// out = dR/d(field)^T v (field space)
    void MultTranspose(const double* v, double* out, cudaStream_t s = nullptr) const { f_->jvp_transpose(v, out, s); }
    int wrt() const { return f_->wrt_; }

   private:
    Functional* f_;
  };

  explicit Functional(const Mesh& mesh) : mesh_(mesh), grad_(this) {
    static_assert(c == 3, "multi-field residuals have a 3-component test space");
    sfx_form h = mesh.create(p, c, false);
    form_ = std::shared_ptr<sfx_form_s>(h, [](sfx_form x) { sfx_form_destroy(x); });
    check(sfx_form_get_layout(h, &L_));
    out_.resize(size_t(L_.num_dofs));
    int cmax = c;
    for (int k = 0; k < nfields; k++) cmax = std::max(cmax, comps_[k]);
    e_.resize(size_t(L_.num_elements) * NPE * size_t(cmax));
  }
  int64_t num_nodes() const { return L_.num_nodes; }

  template <int... i, typename QF>
  void AddDomainIntegral(Dimension<3>, DependsOn<i...>, const QF& qf) {
    static_assert(sizeof...(i) >= 1 && sizeof...(i) <= 4, "one to four arguments");
    static_assert(((i >= 0 && i < nfields) && ...), "DependsOn index out of range");
    using Pos = tuple<tensor<double, 3>, tensor<double, 3, 3>>;
    if constexpr (std::is_invocable<const QF&, double, Pos,
                                    tuple<kernels::value_t<comps_[i], double>, kernels::grad_t<comps_[i], double>>...>::value)
      integrals_.emplace_back(new detail::MultiIntegral<p, c, QF, Nothing, Comps, i...>(qf));
    else
      integrals_.emplace_back(new detail::MultiIntegral<p, c, QF, Empty, Comps, i...>(qf));
  }

  /// R(t, fields...) into a member buffer
  template <typename... F>
  auto operator()(double t, const F&... fields) {
    static_assert(sizeof...(F) == size_t(nfields), "one argument per trial field");
    const double* ptr[nfields] = {field_ptr(fields)...};
    residual(t, ptr, out_.p, nullptr);
    constexpr int nwrt = (0 + ... + int(std::is_same<F, differentiate_wrt_this>::value));
    static_assert(nwrt <= 1, "differentiate with respect to one argument at a time");
    if constexpr (nwrt == 0) {
      return static_cast<const double*>(out_.p);
    } else {
      int k = 0, w = -1;
      ((std::is_same<F, differentiate_wrt_this>::value ? (w = k, k++) : k++), ...);
      linearize(t, ptr, w, nullptr);
      return std::tuple<const double*, Gradient&>{out_.p, grad_};
    }
  }
  void residual(double t, const double* const* fields, double* r, cudaStream_t s) {
    if (integrals_.empty()) throw std::runtime_error("sfx: no integrals");
    for (size_t n = 0; n < integrals_.size(); n++) {
      integrals_[n]->residual(L_, t, fields, e_.p, s);
      detail::scatter_c<c, NPE>(L_, e_.p, r, n > 0, s);
    }
  }
  void linearize(double t, const double* const* fields, int wrt, cudaStream_t s) {
    if (wrt < 0 || wrt >= nfields) throw std::runtime_error("sfx: no such trial field");
    depends_.assign(integrals_.size(), false);
    for (size_t n = 0; n < integrals_.size(); n++) depends_[n] = integrals_[n]->linearize(L_, t, fields, wrt, s);
    wrt_ = wrt;
  }

 private:
  friend class Gradient;
  static const double* field_ptr(const double* u) { return u; }
  static const double* field_ptr(const differentiate_wrt_this& w) { return w.u; }
  void jvp(const double* d, double* df, cudaStream_t s) {
    if (wrt_ < 0) throw std::runtime_error("sfx: linearise first");
    bool first = true;
    for (size_t n = 0; n < integrals_.size(); n++) {
      if (!depends_[n]) continue;
      integrals_[n]->jvp(L_, d, e_.p, s);
      detail::scatter_c<c, NPE>(L_, e_.p, df, !first, s);
      first = false;
    }
    if (first) check_cuda(cudaMemsetAsync(df, 0, sizeof(double) * size_t(L_.num_dofs), s), "memset");
  }
  void jvp_transpose(const double* v, double* out, cudaStream_t s) {
    if (wrt_ < 0) throw std::runtime_error("sfx: linearise first");
    const int cw = comps_[wrt_];
    bool first = true;
    for (size_t n = 0; n < integrals_.size(); n++) {
      if (!depends_[n]) continue;
      integrals_[n]->jvp_transpose(L_, v, e_.p, s);
      if (cw == 1) detail::scatter_c<1, NPE>(L_, e_.p, out, !first, s);
      else detail::scatter_c<3, NPE>(L_, e_.p, out, !first, s);
      first = false;
    }
    if (first) check_cuda(cudaMemsetAsync(out, 0, sizeof(double) * size_t(L_.num_nodes * cw), s), "memset");
  }

  Mesh mesh_;
  std::shared_ptr<sfx_form_s> form_;
  sfx_form_layout L_{};
  Gradient grad_;
  DeviceArray<double> out_, e_;
  std::vector<std::unique_ptr<detail::MultiIntegralBase>> integrals_;
  std::vector<bool> depends_;
  int wrt_ = -1;
};

/// Functional<double(H1<p,c>)>: a quantity of interest (functional_qoi.inl:58-528)
/// over user q-functions qf(t, tuple{X, dX/dxi}, tuple{u, du/dX}) -> scalar
/// (domain) and qf(t, tuple{X, dX/d(s,t)}, tuple{u, du/d(s,t)}) -> scalar
/// (box sides).  Q(t, u) = operator()(t, u); (Q, dQ/du) =
/// operator()(t, differentiate_wrt(u)) with dQ/du(dx) the directional
/// derivative (functional_qoi.inl:420) and assemble(dQ/du) the gradient
/// vector (:422-475, a device buffer of the functional).  Values reduce in a
/// fixed order (deterministic).
template <int p, int c>
class Functional<double(H1<p, c>)> {
 public:
  class Gradient {
   public:
    explicit Gradient(Functional* f) : f_(f) {}
    /// dQ/du(t_lin, u_lin) dx (synchronises to return a host value)
    double operator()(const double* dx, cudaStream_t s = nullptr) const { return f_->action(dx, s); }
    /// the same into a device double
    void Action(const double* dx, double* value, cudaStream_t s = nullptr) const { f_->action_device(dx, value, s); }
    /// dQ/du as a device vector (a member buffer overwritten by the next call)
    const double* assemble(cudaStream_t s = nullptr) { return f_->gradient(s); }
    friend const double* assemble(Gradient& g) { return g.assemble(); }

   private:
    Functional* f_;
  };

  explicit Functional(const Mesh& mesh) : mesh_(mesh), grad_(this) {
    sfx_form h = mesh.create(p, c, true);
    form_ = std::shared_ptr<sfx_form_s>(h, [](sfx_form x) { sfx_form_destroy(x); });
    check(sfx_form_get_layout(h, &L_));
    g_.resize(size_t(L_.num_dofs));
    u_lin_.resize(size_t(L_.num_dofs));
    value_.resize(1);
    partial_.resize(size_t(kernels::kQoiMaxPartials));
  }

  int64_t num_dofs() const { return L_.num_dofs; }

  /// AddDomainIntegral (functional_qoi.inl:159-189)
  template <typename QF>
  void AddDomainIntegral(Dimension<3>, DependsOn<0>, const QF& qf) {
    integrals_.emplace_back(new detail::QoiDomain<p, c, QF>(qf));
  }
  /// AddBoundaryIntegral over the box sides in side_mask (functional_qoi.inl:201-228)
  template <typename QF>
  void AddBoundaryIntegral(Dimension<2>, DependsOn<0>, const QF& qf, int side_mask) {
    auto h = std::make_unique<detail::QoiFaces<p, c, QF>>(qf);
    check(sfx_form_add_face_set(form_.get(), side_mask, &h->face_set));
    check(sfx_form_get_face_layout(form_.get(), h->face_set, &h->F));
    integrals_.push_back(std::move(h));
  }
  /// the same over a face list (element, local side 1..6)
  template <typename QF>
  void AddBoundaryIntegral(Dimension<2>, DependsOn<0>, const QF& qf, const std::vector<int32_t>& face_elem,
                           const std::vector<int32_t>& face_side) {
    if (face_elem.size() != face_side.size()) throw std::runtime_error("sfx: face lists differ in length");
    auto h = std::make_unique<detail::QoiFaces<p, c, QF>>(qf);
    check(sfx_form_add_face_set_faces(form_.get(), int64_t(face_elem.size()), face_elem.data(), face_side.data(),
                                      &h->face_set));
    check(sfx_form_get_face_layout(form_.get(), h->face_set, &h->F));
    integrals_.push_back(std::move(h));
  }
  /// evaluate on X + shape (device, 3 * num_nodes doubles; nullptr = none)
  void SetShapeDisplacement(const double* shape, cudaStream_t s = nullptr) {
    check(sfx_form_set_shape_displacement(form_.get(), shape, s));
    check(sfx_form_get_layout(form_.get(), &L_));  // the shape field's device address
  }
  /// dQ/dp (t, u; p) into out (device, 3 * num_nodes doubles)
  void ShapeGradient(double t, const double* u, double* out, cudaStream_t s = nullptr) {
    if (integrals_.empty()) throw std::runtime_error("sfx: no integrals");
    e3_.resize(size_t(L_.num_elements) * size_t((p + 1) * (p + 1) * (p + 1)) * 3);
    check_cuda(cudaMemsetAsync(out, 0, sizeof(double) * size_t(3 * L_.num_nodes), s), "memset");
    for (auto& in : integrals_) in->shape_gradient(L_, t, u, e3_.p, out, s);
  }

  /// Q(t, u) into a device double
  void Evaluate(double t, const double* u, double* value, cudaStream_t s = nullptr) {
    run(kernels::QOI_VALUE, t, u, nullptr, nullptr, value, s);
  }
  /// Q(t, u) (synchronises)
  double operator()(double t, const double* u, cudaStream_t s = nullptr) {
    Evaluate(t, u, value_.p, s);
    return read_value(s);
  }
  /// (Q(t, u), dQ/du at u)
  std::tuple<double, Gradient&> operator()(double t, differentiate_wrt_this w, cudaStream_t s = nullptr) {
    check_cuda(cudaMemcpyAsync(u_lin_.p, w.u, sizeof(double) * size_t(L_.num_dofs), cudaMemcpyDeviceToDevice, s),
               "copy u");
    t_lin_ = t;
    linearized_ = true;
    Evaluate(t, u_lin_.p, value_.p, s);
    return {read_value(s), grad_};
  }

 private:
  friend class Gradient;
  void run(int mode, double t, const double* u, const double* du, double* grad, double* value, cudaStream_t s) {
    if (integrals_.empty()) throw std::runtime_error("sfx: no integrals");
    int64_t n = 0;
    for (auto& in : integrals_) n += in->count(L_);
    if (vals_.n < size_t(n)) vals_.resize(size_t(n));
    if (grad) check_cuda(cudaMemsetAsync(grad, 0, sizeof(double) * size_t(L_.num_dofs), s), "memset");
    int64_t at = 0;
    for (auto& in : integrals_) {
      in->run(mode, L_, form_.get(), t, u, du, vals_.p + at, grad, s);
      at += in->count(L_);
    }
    if (value) {
      if (n == 0) check_cuda(cudaMemsetAsync(value, 0, sizeof(double), s), "memset");
      else check_cuda(kernels::qoi_sum(vals_.p, n, partial_.p, value, s), "QoI sum");
    }
  }
  double read_value(cudaStream_t s) {
    double v = 0.0;
    check_cuda(cudaMemcpyAsync(&v, value_.p, sizeof(double), cudaMemcpyDeviceToHost, s), "read value");
    check_cuda(cudaStreamSynchronize(s), "synchronise");
    return v;
  }
  void require_linearized() const {
    if (!linearized_) throw std::runtime_error("sfx: differentiate with operator()(t, differentiate_wrt(u)) first");
  }
  void action_device(const double* dx, double* value, cudaStream_t s) {
    require_linearized();
    run(kernels::QOI_ACTION, t_lin_, u_lin_.p, dx, nullptr, value, s);
  }
  double action(const double* dx, cudaStream_t s) {
    action_device(dx, value_.p, s);
    return read_value(s);
  }
  const double* gradient(cudaStream_t s) {
    require_linearized();
    run(kernels::QOI_GRADIENT, t_lin_, u_lin_.p, nullptr, g_.p, nullptr, s);
    return g_.p;
  }

  Mesh mesh_;
  std::shared_ptr<sfx_form_s> form_;
  sfx_form_layout L_{};
  std::vector<std::unique_ptr<detail::QoiBase>> integrals_;
  DeviceArray<double> g_, u_lin_, value_, partial_, vals_, e3_;
  double t_lin_ = 0.0;
  bool linearized_ = false;
  Gradient grad_;
};

/// ShapeAwareFunctional<H1<p,3>, H1<p,c>(H1<p,c>)> (shape_aware_functional.hpp:330-560):
/// the shape displacement comes first after time and is held fixed by the
/// evaluation; r = f(t, shape, u), (r, dR/du) = f(t, shape, differentiate_wrt(u)).
template <typename Shape, typename Sig>
class ShapeAwareFunctional;

template <int p, int c>
class ShapeAwareFunctional<H1<p, 3>, H1<p, c>(H1<p, c>)> : public Functional<H1<p, c>(H1<p, c>)> {
  using Base = Functional<H1<p, c>(H1<p, c>)>;

 public:
  using Base::Base;
  using Base::operator();
  const double* operator()(double t, const double* shape, const double* u, cudaStream_t s = nullptr) {
    Base::SetShapeDisplacement(shape, s);
    return Base::operator()(t, u, s);
  }
  std::tuple<const double*, typename Base::Gradient&> operator()(double t, const double* shape,
                                                                 differentiate_wrt_this w, cudaStream_t s = nullptr) {
    Base::SetShapeDisplacement(shape, s);
    return Base::operator()(t, w, s);
  }
};

}  // namespace sfx
