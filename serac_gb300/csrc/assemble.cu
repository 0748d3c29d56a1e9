// CSR graph, element-stiffness assembly and diagonal of dR/du
// (serac: Gradient::assemble, functional.hpp:569-667; GradientAssemblyLookupTables,
// dof_numbering.hpp:290-351).  Deterministic: one thread owns each row and adds
// its elements' contributions in element order.
#include <cuda_runtime.h>

#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <string>
#include <vector>

#include "dispatch.hpp"
#include "form.hpp"
#include "graph.hpp"
#include "sfx.h"
#include "sfx/kernels.cuh"

using namespace sfx_impl;

namespace {

// scalar adjacency of an imported element table: for every node, the sorted
// union of the nodes of its elements (host build, uploaded once)
int build_table_adjacency(sfx_form f) {
  const int64_t nn = f->nnodes;
  const int NPE = f->NPE;
  std::vector<int32_t> count(size_t(nn) + 1, 0);
  for (int32_t node : f->conn_host) count[size_t(node) + 1]++;
  for (size_t i = 1; i < count.size(); i++) count[i] += count[i - 1];
  std::vector<int32_t> elems(f->conn_host.size());
  {
    std::vector<int32_t> fill(count.begin(), count.end() - 1);
    for (size_t k = 0; k < f->conn_host.size(); k++) elems[size_t(fill[size_t(f->conn_host[k])]++)] = int32_t(k / NPE);
  }
  std::vector<int64_t> sptr(size_t(nn) + 1, 0);
  std::vector<int32_t> scol;
  scol.reserve(size_t(nn) * 27);
  std::vector<int64_t> mark(size_t(nn), -1);
  std::vector<int32_t> row;
  for (int64_t n = 0; n < nn; n++) {
    row.clear();
    for (int32_t t = count[size_t(n)]; t < count[size_t(n) + 1]; t++) {
      const int64_t e = elems[size_t(t)];
      for (int b = 0; b < NPE; b++) {
        const int32_t m = f->conn_host[size_t(e * NPE + b)];
        if (mark[size_t(m)] != n) {
          mark[size_t(m)] = n;
          row.push_back(m);
        }
      }
    }
    std::sort(row.begin(), row.end());
    scol.insert(scol.end(), row.begin(), row.end());
    sptr[size_t(n) + 1] = int64_t(scol.size());
  }
  cudaError_t err;
  if ((err = f->sptr.upload(sptr.data(), sptr.size())) != cudaSuccess ||
      (err = f->scol.upload(scol.data(), scol.size())) != cudaSuccess)
    return fail(SFX_ERR_CUDA, std::string("graph upload: ") + cudaGetErrorString(err));
  return SFX_OK;
}

int build_graph(sfx_form f, cudaStream_t s) {
  if (f->csr_built) return SFX_OK;
  if (f->general && !f->sptr.p)
    if (int rc = build_table_adjacency(f)) return rc;
  const int64_t rows = f->ndofs;
  SFX_CUDA_TRY(f->row_ptr.alloc(size_t(rows + 1)));
  const unsigned blocks = unsigned((rows + 255) / 256);
  with_graph(*f, [&](auto g) {
    if (f->c == 1) sfx::kernels::csr_row_length_kernel<1><<<blocks, 256, 0, s>>>(g, f->row_ptr.p);
    else sfx::kernels::csr_row_length_kernel<3><<<blocks, 256, 0, s>>>(g, f->row_ptr.p);
    return SFX_OK;
  });
  SFX_CUDA_TRY(cudaGetLastError());
  size_t tmp_bytes = 0;
  SFX_CUDA_TRY(cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, f->row_ptr.p, f->row_ptr.p, rows + 1, s));
  DeviceBuf<char> tmp;
  SFX_CUDA_TRY(tmp.alloc(tmp_bytes));
  SFX_CUDA_TRY(cub::DeviceScan::InclusiveSum(tmp.p, tmp_bytes, f->row_ptr.p, f->row_ptr.p, rows + 1, s));
  int64_t nnz = 0;
  SFX_CUDA_TRY(cudaMemcpyAsync(&nnz, f->row_ptr.p + rows, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  SFX_CUDA_TRY(cudaStreamSynchronize(s));
  if (nnz >= (int64_t(1) << 62)) return fail(SFX_ERR_UNSUPPORTED, "nnz overflow");
  SFX_CUDA_TRY(f->col.alloc(size_t(nnz)));
  with_graph(*f, [&](auto g) {
    if (f->c == 1) sfx::kernels::csr_fill_kernel<1><<<blocks, 256, 0, s>>>(g, f->row_ptr.p, f->col.p);
    else sfx::kernels::csr_fill_kernel<3><<<blocks, 256, 0, s>>>(g, f->row_ptr.p, f->col.p);
    return SFX_OK;
  });
  SFX_CUDA_TRY(cudaGetLastError());
  f->nnz = nnz;
  f->csr_built = true;
  return SFX_OK;
}

template <int P, int C>
int assemble_chunk(sfx_form f, const double* Ke, int64_t e0, int64_t e1, double* values, bool accumulate,
                   cudaStream_t s) {
  const unsigned blocks = unsigned((f->ndofs + 127) / 128);
  with_graph(*f, [&](auto g) {
    sfx::kernels::csr_assemble_kernel<P, C><<<blocks, 128, 0, s>>>(g, f->row_ptr.p, f->conn.p, f->node_ptr.p,
                                                                   f->node_ent.p, Ke, e0, e1, values, accumulate);
    return SFX_OK;
  });
  SFX_CUDA_TRY(cudaGetLastError());
  return SFX_OK;
}

int assemble_dispatch(sfx_form f, const double* Ke, int64_t e0, int64_t e1, double* values, bool accumulate,
                      cudaStream_t s) {
  if (f->p == 1 && f->c == 1) return assemble_chunk<1, 1>(f, Ke, e0, e1, values, accumulate, s);
  if (f->p == 1 && f->c == 3) return assemble_chunk<1, 3>(f, Ke, e0, e1, values, accumulate, s);
  if (f->p == 2 && f->c == 1) return assemble_chunk<2, 1>(f, Ke, e0, e1, values, accumulate, s);
  if (f->p == 2 && f->c == 3) return assemble_chunk<2, 3>(f, Ke, e0, e1, values, accumulate, s);
  return fail(SFX_ERR_UNSUPPORTED, "unsupported (order, components)");
}

// element matrices are produced and assembled in chunks of this many elements
constexpr int64_t kChunkElements = 32768;

}  // namespace

extern "C" {

int sfx_csr_nnz(sfx_form form, int64_t* nnz) {
  if (!form || !nnz) return fail(SFX_ERR_INVALID, "null argument");
  if (int rc = build_graph(form, nullptr)) return rc;
  *nnz = form->nnz;
  return SFX_OK;
}

int sfx_csr_graph(sfx_form form, int64_t* row_ptr, int32_t* col, void* stream) {
  if (!form || !row_ptr || !col) return fail(SFX_ERR_INVALID, "null argument");
  auto s = static_cast<cudaStream_t>(stream);
  if (int rc = build_graph(form, s)) return rc;
  SFX_CUDA_TRY(cudaMemcpyAsync(row_ptr, form->row_ptr.p, size_t(form->ndofs + 1) * sizeof(int64_t),
                               cudaMemcpyDeviceToDevice, s));
  SFX_CUDA_TRY(cudaMemcpyAsync(col, form->col.p, size_t(form->nnz) * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  return SFX_OK;
}

int sfx_assemble_csr(sfx_form form, double* values, void* stream) {
  if (!form || !values) return fail(SFX_ERR_INVALID, "null argument");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_assemble_csr");
  if (form->domain.empty() && form->boundary.empty()) return fail(SFX_ERR_INVALID, "no integrals");
  auto s = static_cast<cudaStream_t>(stream);
  if (int rc = build_graph(form, s)) return rc;
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(values, 0, sizeof(double) * size_t(form->nnz), s));
  const int64_t ndof_e = int64_t(form->NPE) * form->c;
  const int64_t chunk = std::min<int64_t>(form->ne, kChunkElements);
  if (form->ke.n < size_t(chunk * ndof_e * ndof_e)) SFX_CUDA_TRY(form->ke.alloc(size_t(chunk * ndof_e * ndof_e)));
  bool first = true;
  for (auto& di : form->domain) {
    for (int64_t e0 = 0; e0 < form->ne; e0 += chunk) {
      const int64_t e1 = std::min(form->ne, e0 + chunk);
      if (int rc = launch_element_matrix(*form, di, false, form->ke.p, e0, e1, s)) return rc;
      if (int rc = assemble_dispatch(form, form->ke.p, e0, e1, values, !first, s)) return rc;
      first = false;
    }
  }
  return assemble_boundary(*form, values, nullptr, s);
}

int sfx_assemble_diagonal(sfx_form form, double* diag, void* stream) {
  if (!form || !diag) return fail(SFX_ERR_INVALID, "null argument");
  if (!form->linearized) return fail(SFX_ERR_INVALID, "sfx_linearize must be called before sfx_assemble_diagonal");
  if (form->domain.empty() && form->boundary.empty()) return fail(SFX_ERR_INVALID, "no integrals");
  auto s = static_cast<cudaStream_t>(stream);
  if (form->domain.empty()) SFX_CUDA_TRY(cudaMemsetAsync(diag, 0, sizeof(double) * size_t(form->ndofs), s));
  for (size_t i = 0; i < form->domain.size(); i++) {
    const auto& di = form->domain[i];
    const bool stored = form->jvp_mode == SFX_JVP_STORED_TANGENT && di.D64.p != nullptr;
    int rc0 = stored ? launch_diag_from_tangent(*form, di, form->e64.p, s)
                     : launch_element_matrix(*form, di, true, form->e64.p, 0, form->ne, s);
    if (rc0) return rc0;
    if (int rc = scatter_evector(*form, form->e64.p, diag, i > 0, s)) return rc;
  }
  return assemble_boundary(*form, nullptr, diag, s);
}

}  // extern "C"
