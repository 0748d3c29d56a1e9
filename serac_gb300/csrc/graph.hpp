// CSR graph of a form: analytic for structured meshes, an explicit scalar
// adjacency for forms built from an imported element table.
#pragma once

#include "form.hpp"
#include "sfx/kernels.cuh"

namespace sfx_impl {

inline sfx::kernels::GridShape grid_shape(const sfx_form_s& f) {
  sfx::kernels::GridShape g{};
  g.p = f.p;
  g.ne[0] = f.mesh.nx;
  g.ne[1] = f.mesh.ny;
  g.ne[2] = f.mesh.nz;
  for (int d = 0; d < 3; d++) g.N[d] = int64_t(f.p) * g.ne[d] + 1;
  return g;
}

inline sfx::kernels::TableGraph table_graph(const sfx_form_s& f) { return {f.sptr.p, f.scol.p, f.nnodes}; }

/// fn(graph) with the form's graph type (the table graph must have been built)
template <typename Fn>
int with_graph(const sfx_form_s& f, Fn&& fn) {
  if (f.general) return fn(table_graph(f));
  return fn(grid_shape(f));
}

}  // namespace sfx_impl
