// sfx C ABI: meshes, forms, residual, linearisation and Jacobian actions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dispatch.hpp"
#include "form.hpp"
#include "sfx.h"
#include "sfx/kernels.cuh"

namespace sfx_impl {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

namespace {

template <int C, int NPE, typename Real>
int scatter(const sfx_form_s& f, const Real* E, Real* out, bool accumulate, cudaStream_t s, int64_t n0 = 0,
            int64_t n1 = -1) {
  if (n1 < 0) n1 = f.nnodes;
  if (n1 <= n0) return SFX_OK;
  constexpr int P = NPE == 8 ? 1 : 2;
  if (!f.general && f.mesh.nx > 0) {
    // structured mesh: whole node planes through the grid scatter (no node -> element table)
    const int Nx = P * f.mesh.nx + 1, Ny = P * f.mesh.ny + 1;
    const int64_t plane = int64_t(Nx) * Ny;
    if (n0 % plane == 0 && n1 % plane == 0) {
      const dim3 grid{unsigned((Nx + 31) / 32), unsigned((Ny + 7) / 8), unsigned((n1 - n0) / plane)};
      sfx::kernels::grid_scatter_kernel<P, C, Real>
          <<<grid, 256, 0, s>>>(E, out, f.mesh.nx, f.mesh.ny, f.mesh.nz, accumulate, int(n0 / plane));
      cudaError_t err = cudaGetLastError();
      if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("scatter launch: ") + cudaGetErrorString(err));
      return SFX_OK;
    }
  }
  unsigned blocks = unsigned((n1 - n0 + 255) / 256);
  sfx::kernels::scatter_kernel<C, NPE, Real>
      <<<blocks, 256, 0, s>>>(E, f.node_ptr.p, f.node_ent.p, out, f.nnodes, accumulate, n0, n1);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("scatter launch: ") + cudaGetErrorString(err));
  return SFX_OK;
}

template <typename Real>
int scatter_dispatch(const sfx_form_s& f, const Real* E, Real* out, bool accumulate, cudaStream_t s) {
  if (f.p == 1 && f.c == 1) return scatter<1, 8, Real>(f, E, out, accumulate, s);
  if (f.p == 1 && f.c == 3) return scatter<3, 8, Real>(f, E, out, accumulate, s);
  if (f.p == 2 && f.c == 1) return scatter<1, 27, Real>(f, E, out, accumulate, s);
  if (f.p == 2 && f.c == 3) return scatter<3, 27, Real>(f, E, out, accumulate, s);
  return fail(SFX_ERR_UNSUPPORTED, "unsupported (order, components)");
}

__global__ void f64_to_f32(const double* a, float* b, int64_t n) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] = float(a[i]);
}

int check_form(sfx_form f) {
  if (!f) return fail(SFX_ERR_INVALID, "null form");
  return SFX_OK;
}

}  // namespace

int scatter_evector(const sfx_form_s& f, const double* E, double* out, bool accumulate, cudaStream_t s) {
  return scatter_dispatch<double>(f, E, out, accumulate, s);
}

int scatter_evector_range(const sfx_form_s& f, const double* E, double* out, int64_t n0, int64_t n1,
                          cudaStream_t s) {
  if (f.p == 1 && f.c == 1) return scatter<1, 8, double>(f, E, out, false, s, n0, n1);
  if (f.p == 1 && f.c == 3) return scatter<3, 8, double>(f, E, out, false, s, n0, n1);
  if (f.p == 2 && f.c == 1) return scatter<1, 27, double>(f, E, out, false, s, n0, n1);
  if (f.p == 2 && f.c == 3) return scatter<3, 27, double>(f, E, out, false, s, n0, n1);
  return fail(SFX_ERR_UNSUPPORTED, "unsupported (order, components)");
}

int scatter_evector3(const sfx_form_s& f, const double* E, double* out, bool accumulate, cudaStream_t s) {
  if (f.p == 1) return scatter<3, 8, double>(f, E, out, accumulate, s);
  if (f.p == 2) return scatter<3, 27, double>(f, E, out, accumulate, s);
  return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
}

int ensure_shape_scratch(sfx_form_s& f) {
  const size_t ne = size_t(f.ne) * size_t(f.NPE) * 3;
  if (f.eshape.n < ne && f.eshape.alloc(ne) != cudaSuccess) return fail(SFX_ERR_NOMEM, "shape scratch");
  size_t nf = 0;
  const size_t npf = size_t(f.p + 1) * size_t(f.p + 1) * 3;
  for (const auto& bi : f.boundary) nf = std::max(nf, size_t(bi.num_faces) * npf);
  for (const auto& bi : f.qoi_boundary) nf = std::max(nf, size_t(bi.num_faces) * npf);
  if (f.efshape.n < nf && f.efshape.alloc(nf) != cudaSuccess) return fail(SFX_ERR_NOMEM, "face shape scratch");
  return SFX_OK;
}

}  // namespace sfx_impl

using namespace sfx_impl;

namespace sfx_impl {
// geometric factors of the domain (and of every boundary integral) in the
// reference configuration, or shape-displaced by f.shape when f.has_shape
int compute_geometry(sfx_form_s& f, cudaStream_t s) {
  const int64_t nqt = f.ne * f.NQ;
  const unsigned blocks = unsigned((nqt + 255) / 256);
  if (f.has_shape) {
    if (f.p == 1)
      sfx::kernels::geometry_shape_kernel<1><<<blocks, 256, 0, s>>>(f.Xe.p, f.conn.p, f.shape.p, f.nnodes, f.geom64.p,
                                                                    f.geom32.p, f.ne);
    else
      sfx::kernels::geometry_shape_kernel<2><<<blocks, 256, 0, s>>>(f.Xe.p, f.conn.p, f.shape.p, f.nnodes, f.geom64.p,
                                                                    f.geom32.p, f.ne);
  } else {
    if (f.Q == 2) sfx::kernels::geometry_kernel<2><<<blocks, 256, 0, s>>>(f.Xe.p, f.geom64.p, f.geom32.p, f.ne);
    else sfx::kernels::geometry_kernel<3><<<blocks, 256, 0, s>>>(f.Xe.p, f.geom64.p, f.geom32.p, f.ne);
  }
  for (auto& bi : f.boundary)
    if (int rc = compute_face_geometry(f, bi, s)) return rc;
  for (auto& bi : f.face_sets)
    if (int rc = compute_face_geometry(f, bi, s)) return rc;
  for (auto& bi : f.qoi_boundary)
    if (int rc = compute_face_geometry(f, bi, s)) return rc;
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}
// every element of an imported table positively oriented in its
// lexicographic frame: the trilinear map's Jacobian at the element centre
// (the mean of the four edges along each of xi, eta, zeta) has a positive
// determinant.  A wrong node or corner permutation inverts the whole element,
// which this catches; mildly distorted elements that serac accepts pass.
// Xe: [e][3][8].
int check_orientation(const std::vector<double>& Xe, int64_t ne) {
  for (int64_t e = 0; e < ne; e++) {
    const double* X = &Xe[size_t(e * 24)];
    double Jc[3][3] = {};
    for (int d = 0; d < 3; d++) {
      const int bit = 1 << d;
      for (int v = 0; v < 8; v++) {
        if (v & bit) continue;
        for (int i = 0; i < 3; i++) Jc[i][d] += 0.25 * (X[i * 8 + (v | bit)] - X[i * 8 + v]);
      }
    }
    const double det = Jc[0][0] * (Jc[1][1] * Jc[2][2] - Jc[1][2] * Jc[2][1]) -
                       Jc[0][1] * (Jc[1][0] * Jc[2][2] - Jc[1][2] * Jc[2][0]) +
                       Jc[0][2] * (Jc[1][0] * Jc[2][1] - Jc[1][1] * Jc[2][0]);
    if (!(det > 0.0))
      return fail(SFX_ERR_INVALID, "element " + std::to_string(e) +
                                       " is inverted or degenerate (non-positive Jacobian at its centre; check the "
                                       "lexicographic node and corner order)");
  }
  return SFX_OK;
}

// sizes, node -> element map, device tables and geometric factors of a new
// form from its element table conn [e][NPE] and vertex coordinates Xe [e][3][8]
int init_form(sfx_form_s* f, int order, int components, int64_t ne, int64_t nnodes, const std::vector<int32_t>& conn,
              const std::vector<double>& Xe) {
  f->p = order;
  f->c = components;
  f->Q = order + 1;
  f->NQ = f->Q * f->Q * f->Q;
  f->NPE = (order + 1) * (order + 1) * (order + 1);
  f->ne = ne;
  f->nnodes = nnodes;
  f->ndofs = nnodes * components;
  std::vector<int32_t> count(size_t(nnodes) + 1, 0);
  for (int32_t node : conn) count[size_t(node) + 1]++;
  for (size_t i = 1; i < count.size(); i++) count[i] += count[i - 1];
  std::vector<int32_t> ent(conn.size());
  {
    std::vector<int32_t> fill(count.begin(), count.end() - 1);
    for (size_t k = 0; k < conn.size(); k++) ent[size_t(fill[size_t(conn[k])]++)] = int32_t(k);
  }
  cudaError_t err;
  if ((err = f->wait_error.init()) != cudaSuccess || (err = f->conn.upload(conn.data(), conn.size())) != cudaSuccess ||
      (err = f->node_ptr.upload(count.data(), count.size())) != cudaSuccess ||
      (err = f->node_ent.upload(ent.data(), ent.size())) != cudaSuccess)
    return fail(SFX_ERR_CUDA, std::string("upload tables: ") + cudaGetErrorString(err));
  const int64_t nqt = f->ne * f->NQ;
  if ((err = f->Xe.upload(Xe.data(), Xe.size())) != cudaSuccess ||
      (err = f->geom64.alloc(size_t(nqt) * sfx::kernels::GEOM_STRIDE)) != cudaSuccess ||
      (err = f->geom32.alloc(size_t(nqt) * sfx::kernels::GEOM_STRIDE)) != cudaSuccess ||
      (err = f->e64.alloc(size_t(f->ne) * f->NPE * components)) != cudaSuccess ||
      (err = f->e32.alloc(size_t(f->ne) * f->NPE * components)) != cudaSuccess ||
      (err = f->u_lin64.alloc(size_t(f->ndofs))) != cudaSuccess ||
      (err = f->u_lin32.alloc(size_t(f->ndofs))) != cudaSuccess)
    return fail(SFX_ERR_NOMEM, std::string("device allocation: ") + cudaGetErrorString(err));
  if (int rc = compute_geometry(*f, nullptr)) return rc;
  if ((err = cudaDeviceSynchronize()) != cudaSuccess)
    return fail(SFX_ERR_CUDA, std::string("geometry kernel: ") + cudaGetErrorString(err));
  return SFX_OK;
}
}  // namespace sfx_impl

extern "C" {

const char* sfx_last_error(void) { return g_last_error.c_str(); }

int sfx_version(void) { return 1; }

int sfx_mesh_create_structured_hex(int nx, int ny, int nz, const double* vertices, sfx_mesh* out) {
  if (!out) return fail(SFX_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (nx < 1 || ny < 1 || nz < 1) return fail(SFX_ERR_INVALID, "mesh dimensions must be >= 1");
  if (!vertices) return fail(SFX_ERR_INVALID, "null vertex array");
  int64_t nv = int64_t(nx + 1) * (ny + 1) * (nz + 1);
  if (int64_t(nx) * ny * nz * 27 >= (int64_t(1) << 31)) return fail(SFX_ERR_UNSUPPORTED, "mesh too large for int32 tables");
  auto* m = new (std::nothrow) sfx_mesh_s;
  if (!m) return fail(SFX_ERR_NOMEM, "host allocation failed");
  m->nx = nx;
  m->ny = ny;
  m->nz = nz;
  m->vertices.assign(vertices, vertices + nv * 3);
  *out = m;
  return SFX_OK;
}

int sfx_mesh_destroy(sfx_mesh mesh) {
  delete mesh;
  return SFX_OK;
}

int sfx_mesh_num_elements(sfx_mesh mesh, int64_t* out) {
  if (!mesh || !out) return fail(SFX_ERR_INVALID, "null argument");
  *out = int64_t(mesh->nx) * mesh->ny * mesh->nz;
  return SFX_OK;
}

int sfx_form_create(sfx_mesh mesh, int order, int components, sfx_form* out) {
  if (!mesh || !out) return fail(SFX_ERR_INVALID, "null argument");
  *out = nullptr;
  if (order < 1 || order > 2) return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
  if (components != 1 && components != 3) return fail(SFX_ERR_UNSUPPORTED, "components must be 1 or 3");
  auto* f = new (std::nothrow) sfx_form_s;
  if (!f) return fail(SFX_ERR_NOMEM, "host allocation failed");
  f->mesh = *mesh;
  const int nx = mesh->nx, ny = mesh->ny, nz = mesh->nz, p = order, n = order + 1;
  const int64_t Nx = int64_t(p) * nx + 1, Ny = int64_t(p) * ny + 1, Nz = int64_t(p) * nz + 1;
  const int64_t ne = int64_t(nx) * ny * nz, npe = int64_t(n) * n * n;
  // element -> node table (lexicographic local order)
  std::vector<int32_t> conn(size_t(ne * npe));
  for (int64_t e = 0; e < ne; e++) {
    int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / (int64_t(nx) * ny);
    for (int kz = 0; kz < n; kz++)
      for (int ky = 0; ky < n; ky++)
        for (int kx = 0; kx < n; kx++) {
          int64_t node = (p * ex + kx) + Nx * ((p * ey + ky) + Ny * (p * ez + kz));
          conn[size_t(e * npe + kx + n * (ky + n * kz))] = int32_t(node);
        }
  }
  // element vertex coordinates [e][3][8]
  std::vector<double> Xe(size_t(ne) * 24);
  for (int64_t e = 0; e < ne; e++) {
    int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / (int64_t(nx) * ny);
    for (int v = 0; v < 8; v++) {
      int64_t vid = (ex + (v & 1)) + int64_t(nx + 1) * ((ey + ((v >> 1) & 1)) + int64_t(ny + 1) * (ez + ((v >> 2) & 1)));
      for (int i = 0; i < 3; i++) Xe[size_t(e * 24 + i * 8 + v)] = mesh->vertices[size_t(vid * 3 + i)];
    }
  }
  if (int rc = sfx_impl::init_form(f, order, components, ne, Nx * Ny * Nz, conn, Xe)) {
    delete f;
    return rc;
  }
  *out = f;
  return SFX_OK;
}

int sfx_form_create_from_table(int order, int components, int64_t num_elements, int64_t num_nodes,
                               const int32_t* elem_nodes, const double* elem_vertices, sfx_form* out) {
  if (!out) return fail(SFX_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (order < 1 || order > 2) return fail(SFX_ERR_UNSUPPORTED, "order must be 1 or 2");
  if (components != 1 && components != 3) return fail(SFX_ERR_UNSUPPORTED, "components must be 1 or 3");
  if (num_elements < 1 || num_nodes < 1) return fail(SFX_ERR_INVALID, "empty element table");
  if (!elem_nodes || !elem_vertices) return fail(SFX_ERR_INVALID, "null table");
  const int64_t npe = int64_t(order + 1) * (order + 1) * (order + 1);
  if (num_elements * npe >= (int64_t(1) << 31) || num_nodes * components >= (int64_t(1) << 31))
    return fail(SFX_ERR_UNSUPPORTED, "table too large for int32 indices");
  std::vector<int32_t> conn(elem_nodes, elem_nodes + num_elements * npe);
  for (int32_t nd : conn)
    if (nd < 0 || nd >= num_nodes) return fail(SFX_ERR_INVALID, "element node id out of range");
  std::vector<double> Xe(size_t(num_elements) * 24);
  for (int64_t e = 0; e < num_elements; e++)
    for (int v = 0; v < 8; v++)
      for (int i = 0; i < 3; i++) Xe[size_t(e * 24 + i * 8 + v)] = elem_vertices[size_t((e * 8 + v) * 3 + i)];
  if (int rc = sfx_impl::check_orientation(Xe, num_elements)) return rc;
  auto* f = new (std::nothrow) sfx_form_s;
  if (!f) return fail(SFX_ERR_NOMEM, "host allocation failed");
  f->general = true;
  if (int rc = sfx_impl::init_form(f, order, components, num_elements, num_nodes, conn, Xe)) {
    delete f;
    return rc;
  }
  f->conn_host = std::move(conn);
  f->Xe_host = std::move(Xe);
  *out = f;
  return SFX_OK;
}

int sfx_form_set_shape_displacement(sfx_form form, const double* shape, void* stream) {
  if (check_form(form)) return fail(SFX_ERR_INVALID, "null form");
  auto st = static_cast<cudaStream_t>(stream);
  if (shape) {
    const size_t n = size_t(3 * form->nnodes);
    if (form->shape.n < n && form->shape.alloc(n) != cudaSuccess) return fail(SFX_ERR_NOMEM, "shape allocation");
    SFX_CUDA_TRY(cudaMemcpyAsync(form->shape.p, shape, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  }
  form->has_shape = shape != nullptr;
  form->linearized = false;  // the stored tangent belongs to the old geometry
  return sfx_impl::compute_geometry(*form, st);
}

int sfx_shape_jvp(sfx_form form, double t, const double* u, const double* dshape, double* dr, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!u || !dshape || !dr) return fail(SFX_ERR_INVALID, "null vector");
  auto s = static_cast<cudaStream_t>(stream);
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(dr, 0, sizeof(double) * size_t(form->ndofs), s));
  for (size_t i = 0; i < form->domain.size(); i++) {
    if (int rc = sfx_impl::launch_shape_jvp(*form, form->domain[i], u, dshape, form->e64.p, t, s)) return rc;
    if (int rc2 = scatter_dispatch<double>(*form, form->e64.p, dr, i > 0, s)) return rc2;
  }
  return sfx_impl::launch_boundary_shape_jvp(*form, u, dshape, dr, t, s);
}

int sfx_shape_vjp(sfx_form form, double t, const double* u, const double* lam, double* out, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!u || !lam || !out) return fail(SFX_ERR_INVALID, "null vector");
  if (form->qoi) return fail(SFX_ERR_INVALID, "a quantity of interest takes sfx_qoi_shape_gradient");
  if (int rc = ensure_shape_scratch(*form)) return rc;
  auto s = static_cast<cudaStream_t>(stream);
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * size_t(3 * form->nnodes), s));
  for (size_t i = 0; i < form->domain.size(); i++) {
    if (int rc = sfx_impl::launch_shape_vjp(*form, form->domain[i], u, lam, form->eshape.p, t, s)) return rc;
    if (int rc2 = scatter_evector3(*form, form->eshape.p, out, i > 0, s)) return rc2;
  }
  return sfx_impl::launch_boundary_shape_vjp(*form, u, lam, out, t, s);
}

int sfx_form_destroy(sfx_form form) {
  delete form;
  return SFX_OK;
}

int sfx_form_num_dofs(sfx_form form, int64_t* out) {
  if (check_form(form) || !out) return fail(SFX_ERR_INVALID, "null argument");
  *out = form->ndofs;
  return SFX_OK;
}

int sfx_form_add_domain_integral(sfx_form form, int material, const double* params, int per_element) {
  if (check_form(form)) return SFX_ERR_INVALID;
  int comps = 0, np = 0, nst = 0;
  if (int rc = material_info(material, &comps, &np, &nst)) return rc;
  if (comps != form->c) return fail(SFX_ERR_INVALID, "material component count does not match the trial space");
  if (form->qoi) return fail(SFX_ERR_INVALID, "a quantity of interest takes sfx_qoi_add_domain_integral");
  if (!form->domain.empty()) return fail(SFX_ERR_UNSUPPORTED, "one domain integral per form in this version");
  if (np > 0 && !params) return fail(SFX_ERR_INVALID, "material needs parameters");
  DomainIntegral di;
  di.material = material;
  di.nparams = np;
  di.state_doubles = nst;
  std::vector<double> prm(size_t(form->ne) * np);
  for (int64_t e = 0; e < form->ne; e++)
    for (int k = 0; k < np; k++) prm[size_t(e * np + k)] = per_element ? params[e * np + k] : params[k];
  cudaError_t err = di.params.upload(prm.data(), prm.size());
  if (err == cudaSuccess && nst > 0) {
    size_t n = size_t(form->ne) * form->NQ * nst;
    err = di.state.alloc(n);
    if (err == cudaSuccess) err = cudaMemset(di.state.p, 0, n * sizeof(double));
  }
  if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("integral setup: ") + cudaGetErrorString(err));
  form->domain.push_back(std::move(di));
  return SFX_OK;
}

int sfx_set_param_field(sfx_form form, int integral, const double* params, int per_element) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (integral < 0 || size_t(integral) >= form->domain.size()) return fail(SFX_ERR_INVALID, "no such domain integral");
  DomainIntegral& di = form->domain[size_t(integral)];
  if (di.nparams == 0) return fail(SFX_ERR_INVALID, "the material takes no parameters");
  if (!params) return fail(SFX_ERR_INVALID, "null parameters");
  std::vector<double> prm(size_t(form->ne) * size_t(di.nparams));
  for (int64_t e = 0; e < form->ne; e++)
    for (int k = 0; k < di.nparams; k++)
      prm[size_t(e * di.nparams + k)] = per_element ? params[e * di.nparams + k] : params[k];
  // work queued on any stream (non-blocking ones included) may still read the
  // old parameters: let it finish before they are overwritten
  SFX_CUDA_TRY(cudaDeviceSynchronize());
  SFX_CUDA_TRY(cudaMemcpy(di.params.p, prm.data(), prm.size() * sizeof(double), cudaMemcpyHostToDevice));
  form->linearized = false;  // the stored tangent belongs to the old parameters
  return SFX_OK;
}

int sfx_residual(sfx_form form, double t, const double* u, double* r, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!u || !r) return fail(SFX_ERR_INVALID, "null vector");
  if (form->domain.empty() && form->boundary.empty()) return fail(SFX_ERR_INVALID, "no integrals");
  auto s = static_cast<cudaStream_t>(stream);
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(r, 0, sizeof(double) * size_t(form->ndofs), s));
  const int mode = form->update_qdata ? sfx::kernels::RESIDUAL_UPDATE : sfx::kernels::RESIDUAL;
  for (size_t i = 0; i < form->domain.size(); i++) {
    if (int rc = launch_domain(*form, form->domain[i], mode, u, nullptr, form->e64.p, t, s)) return rc;
    if (int rc = scatter_dispatch<double>(*form, form->e64.p, r, i > 0, s)) return rc;
  }
  return launch_boundary(*form, sfx::kernels::RESIDUAL, u, nullptr, r, t, s);
}

int sfx_linearize(sfx_form form, double t, const double* u, double* r, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!u) return fail(SFX_ERR_INVALID, "null vector");
  if (form->domain.empty() && form->boundary.empty()) return fail(SFX_ERR_INVALID, "no integrals");
  auto s = static_cast<cudaStream_t>(stream);
  SFX_CUDA_TRY(cudaMemcpyAsync(form->u_lin64.p, u, size_t(form->ndofs) * sizeof(double), cudaMemcpyDeviceToDevice, s));
  unsigned blocks = unsigned((form->ndofs + 255) / 256);
  if (form->ndofs) f64_to_f32<<<blocks, 256, 0, s>>>(form->u_lin64.p, form->u_lin32.p, form->ndofs);
  SFX_CUDA_TRY(cudaGetLastError());
  form->t_lin = t;
  form->linearized = true;
  if (form->jvp_mode == SFX_JVP_STORED_TANGENT) {
    if (r && form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(r, 0, sizeof(double) * size_t(form->ndofs), s));
    for (size_t i = 0; i < form->domain.size(); i++) {
      if (int rc = launch_linearize(*form, form->domain[i], r ? form->e64.p : nullptr, s)) return rc;
      if (r)
        if (int rc = scatter_dispatch<double>(*form, form->e64.p, r, i > 0, s)) return rc;
    }
    if (r) return launch_boundary(*form, sfx::kernels::RESIDUAL, form->u_lin64.p, nullptr, r, t, s);
    return SFX_OK;
  }
  if (r) {
    bool saved = form->update_qdata;
    form->update_qdata = false;
    int rc = sfx_residual(form, t, form->u_lin64.p, r, stream);
    form->update_qdata = saved;
    return rc;
  }
  return SFX_OK;
}

int sfx_form_set_jvp_mode(sfx_form form, int mode) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (mode != SFX_JVP_STORED_TANGENT && mode != SFX_JVP_RECOMPUTE) return fail(SFX_ERR_INVALID, "unknown jvp mode");
  if (mode != form->jvp_mode) form->linearized = false;
  form->jvp_mode = mode;
  return SFX_OK;
}

int sfx_form_set_tangent_storage(sfx_form form, int storage) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (storage != SFX_TANGENT_F32 && storage != SFX_TANGENT_F16) return fail(SFX_ERR_INVALID, "unknown tangent storage");
  if (storage == SFX_TANGENT_F16 && form->p != 2)
    return fail(SFX_ERR_UNSUPPORTED, "the FP16 tangent copy is built for order 2");
  const bool want = storage == SFX_TANGENT_F16;
  if (want != form->tangent16) form->linearized = false;
  form->tangent16 = want;
  return SFX_OK;
}

int sfx_jvp(sfx_form form, const double* du, double* dr, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!du || !dr) return fail(SFX_ERR_INVALID, "null vector");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_jvp");
  auto s = static_cast<cudaStream_t>(stream);
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(dr, 0, sizeof(double) * size_t(form->ndofs), s));
  for (size_t i = 0; i < form->domain.size(); i++) {
    int rc = form->jvp_mode == SFX_JVP_STORED_TANGENT
                 ? launch_jvp_stored(*form, form->domain[i], du, form->e64.p, s)
                 : launch_domain(*form, form->domain[i], sfx::kernels::JVP, form->u_lin64.p, du, form->e64.p,
                                 form->t_lin, s);
    if (rc) return rc;
    if (int rc2 = scatter_dispatch<double>(*form, form->e64.p, dr, i > 0, s)) return rc2;
  }
  return launch_boundary(*form, sfx::kernels::JVP, form->u_lin64.p, du, dr, form->t_lin, s);
}

int sfx_jvp_f32(sfx_form form, const float* du, float* dr, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!du || !dr) return fail(SFX_ERR_INVALID, "null vector");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_jvp_f32");
  if (form->wait_error.raised()) {
    form->wait_error.clear();
    return fail(SFX_ERR_TIMEOUT, "a bulk-copy wait of an earlier FP32 Jacobian action expired");
  }
  auto s = static_cast<cudaStream_t>(stream);
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(dr, 0, sizeof(float) * size_t(form->ndofs), s));
  for (size_t i = 0; i < form->domain.size(); i++) {
    int rc = form->jvp_mode == SFX_JVP_STORED_TANGENT
                 ? launch_jvp_stored_f32(*form, form->domain[i], du, form->e32.p, s)
                 : launch_domain_jvp_f32(*form, form->domain[i], form->u_lin32.p, du, form->e32.p, form->t_lin, s);
    if (rc) return rc;
    if (int rc2 = scatter_dispatch<float>(*form, form->e32.p, dr, i > 0, s)) return rc2;
  }
  return launch_boundary_jvp_f32(*form, form->u_lin32.p, du, dr, form->t_lin, s);
}

int sfx_jvp_transpose(sfx_form form, const double* v, double* dr, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!v || !dr) return fail(SFX_ERR_INVALID, "null vector");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_jvp_transpose");
  if (!form->domain.empty() && form->jvp_mode != SFX_JVP_STORED_TANGENT)
    return fail(SFX_ERR_UNSUPPORTED, "the transposed action needs the stored tangent (SFX_JVP_STORED_TANGENT)");
  auto s = static_cast<cudaStream_t>(stream);
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(dr, 0, sizeof(double) * size_t(form->ndofs), s));
  for (size_t i = 0; i < form->domain.size(); i++) {
    if (int rc = launch_jvp_transpose(*form, form->domain[i], v, form->e64.p, s)) return rc;
    if (int rc2 = scatter_dispatch<double>(*form, form->e64.p, dr, i > 0, s)) return rc2;
  }
  return launch_boundary_transpose(*form, v, dr, s);
}

int sfx_jvp_transpose_f32(sfx_form form, const float* v, float* dr, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!v || !dr) return fail(SFX_ERR_INVALID, "null vector");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_jvp_transpose_f32");
  if (!form->domain.empty() && form->jvp_mode != SFX_JVP_STORED_TANGENT)
    return fail(SFX_ERR_UNSUPPORTED, "the transposed action needs the stored tangent (SFX_JVP_STORED_TANGENT)");
  if (form->wait_error.raised()) {
    form->wait_error.clear();
    return fail(SFX_ERR_TIMEOUT, "a bulk-copy wait of an earlier FP32 Jacobian action expired");
  }
  auto s = static_cast<cudaStream_t>(stream);
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(dr, 0, sizeof(float) * size_t(form->ndofs), s));
  for (size_t i = 0; i < form->domain.size(); i++) {
    if (int rc = launch_jvp_transpose_f32(*form, form->domain[i], v, form->e32.p, s)) return rc;
    if (int rc2 = scatter_dispatch<float>(*form, form->e32.p, dr, i > 0, s)) return rc2;
  }
  return launch_boundary_transpose_f32(*form, v, dr, s);
}

int sfx_jvp_element(sfx_form form, const double* du, double* dE, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!du || !dE) return fail(SFX_ERR_INVALID, "null vector");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_jvp_element");
  if (form->domain.empty()) return fail(SFX_ERR_INVALID, "no domain integral");
  auto s = static_cast<cudaStream_t>(stream);
  if (form->jvp_mode == SFX_JVP_STORED_TANGENT) return launch_jvp_stored(*form, form->domain[0], du, dE, s);
  return launch_domain(*form, form->domain[0], sfx::kernels::JVP, form->u_lin64.p, du, dE, form->t_lin, s);
}

int sfx_jvp_element_f32(sfx_form form, const float* du, float* dE, void* stream) {
  if (check_form(form)) return SFX_ERR_INVALID;
  if (!du || !dE) return fail(SFX_ERR_INVALID, "null vector");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_jvp_element_f32");
  if (form->domain.empty()) return fail(SFX_ERR_INVALID, "no domain integral");
  if (form->wait_error.raised()) {
    form->wait_error.clear();
    return fail(SFX_ERR_TIMEOUT, "a bulk-copy wait of an earlier FP32 Jacobian action expired");
  }
  auto s = static_cast<cudaStream_t>(stream);
  if (form->jvp_mode == SFX_JVP_STORED_TANGENT) return launch_jvp_stored_f32(*form, form->domain[0], du, dE, s);
  return launch_domain_jvp_f32(*form, form->domain[0], form->u_lin32.p, du, dE, form->t_lin, s);
}

int sfx_form_get_layout(sfx_form form, sfx_form_layout* out) {
  if (check_form(form) || !out) return fail(SFX_ERR_INVALID, "null argument");
  sfx_form_layout L{};
  L.order = form->p;
  L.components = form->c;
  L.num_elements = form->ne;
  L.num_nodes = form->nnodes;
  L.num_dofs = form->ndofs;
  L.conn = form->conn.p;
  L.node_ptr = form->node_ptr.p;
  L.node_ent = form->node_ent.p;
  L.geom = form->geom64.p;
  L.geom_f32 = form->geom32.p;
  L.evector = form->e64.p;
  L.evector_f32 = form->e32.p;
  L.row_ptr = form->csr_built ? form->row_ptr.p : nullptr;
  L.nx = form->mesh.nx;
  L.ny = form->mesh.ny;
  L.nz = form->mesh.nz;
  L.general = form->general ? 1 : 0;
  L.graph_ptr = form->sptr.p;
  L.graph_col = form->scol.p;
  L.elem_vertices = form->Xe.p;
  L.shape = form->has_shape ? form->shape.p : nullptr;
  *out = L;
  return SFX_OK;
}

int sfx_scatter_add(sfx_form form, const double* E, double* out, int accumulate, void* stream) {
  if (check_form(form) || !E || !out) return fail(SFX_ERR_INVALID, "null argument");
  return scatter_dispatch<double>(*form, E, out, accumulate != 0, static_cast<cudaStream_t>(stream));
}

int sfx_scatter_add_f32(sfx_form form, const float* E, float* out, int accumulate, void* stream) {
  if (check_form(form) || !E || !out) return fail(SFX_ERR_INVALID, "null argument");
  return scatter_dispatch<float>(*form, E, out, accumulate != 0, static_cast<cudaStream_t>(stream));
}

int sfx_update_qdata(sfx_form form, int flag) {
  if (check_form(form)) return SFX_ERR_INVALID;
  form->update_qdata = flag != 0;
  return SFX_OK;
}

int sfx_qdata_size(sfx_form form, int64_t* num_doubles) {
  if (check_form(form) || !num_doubles) return fail(SFX_ERR_INVALID, "null argument");
  *num_doubles = 0;
  for (auto& di : form->domain) *num_doubles += form->ne * form->NQ * di.state_doubles;
  return SFX_OK;
}

static int qdata_copy(sfx_form form, double* host, bool to_device) {
  for (auto& di : form->domain) {
    if (!di.state_doubles) continue;
    const int64_t nqt = form->ne * form->NQ;
    const int k = di.state_doubles;
    std::vector<double> soa(size_t(nqt) * k);
    if (to_device) {
      for (int64_t q = 0; q < nqt; q++)
        for (int j = 0; j < k; j++) soa[size_t(j * nqt + q)] = host[q * k + j];
      SFX_CUDA_TRY(cudaMemcpy(di.state.p, soa.data(), soa.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else {
      SFX_CUDA_TRY(cudaMemcpy(soa.data(), di.state.p, soa.size() * sizeof(double), cudaMemcpyDeviceToHost));
      for (int64_t q = 0; q < nqt; q++)
        for (int j = 0; j < k; j++) host[q * k + j] = soa[size_t(j * nqt + q)];
    }
    host += nqt * k;
  }
  return SFX_OK;
}

int sfx_set_qdata(sfx_form form, const double* host_state) {
  if (check_form(form) || !host_state) return fail(SFX_ERR_INVALID, "null argument");
  return qdata_copy(form, const_cast<double*>(host_state), true);
}

int sfx_get_qdata(sfx_form form, double* host_state) {
  if (check_form(form) || !host_state) return fail(SFX_ERR_INVALID, "null argument");
  return qdata_copy(form, host_state, false);
}

}  // extern "C"
