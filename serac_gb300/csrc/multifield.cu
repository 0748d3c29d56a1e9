// Multi-field forms of the C ABI: serac's Functional<test(trial_0, ...,
// trial_{n-1})> (functional.hpp:189-317) as SolidMechanics builds it,
// test(displacement, acceleration, parameters...) with materials added under
// DependsOn<0, 1, parameters...> (solid_mechanics.hpp:243, 880-893).
//
// A multi-field form owns a single-field form of the test space (element
// tables, node -> element map, geometric factors, E-vector scratch) and its
// argument fields' component counts.  Residual, derivative storage with
// respect to one field, and the derivative's action and transposed action
// run the kernels of sfx/multifield.cuh; results are summed into the output
// by the deterministic node-owner scatter of the field they belong to.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "form.hpp"
#include "sfx.h"
#include "sfx/materials.hpp"
#include "sfx/multifield.cuh"

using namespace sfx_impl;

namespace {

using namespace sfx;

struct ParamNeoHookeanMaker {
  static constexpr int nparams = 3;  // density, K0, G0
  SFX_HD solid_mechanics::MultiFieldStressFunctor<solid_mechanics::ParameterizedNeoHookean, true> operator()(
      const double* p) const {
    return {solid_mechanics::ParameterizedNeoHookean{p[0], p[1], p[2]}};
  }
};

struct MultiIntegral {
  int material = 0;
  std::vector<int> args;  // form field of each material argument (DependsOn)
  DeviceBuf<double> params;
  DeviceBuf<double> D;  // stored derivative with respect to the argument `lin_arg`
  int lin_arg = -1;     // argument the stored derivative belongs to (-1: none, or the form field is not an argument)
};

}  // namespace

struct sfx_mform_s {
  sfx_form base = nullptr;  // test space: tables, geometry, scatter
  int test_components = 0;
  std::vector<int> comps;  // per form field
  std::vector<MultiIntegral> integrals;
  DeviceBuf<double> E;  // E-vector scratch, NPE x max(components) per element
  int lin_field = -1;   // form field of the current linearisation
  ~sfx_mform_s() {
    if (base) sfx_form_destroy(base);
  }
};

namespace {

int check(sfx_mform f) { return f ? SFX_OK : fail(SFX_ERR_INVALID, "null multi-field form"); }

template <int C, int NPE>
int scatter_c(const sfx_form_s& f, const double* E, double* out, bool accumulate, cudaStream_t s) {
  if (f.nnodes == 0) return SFX_OK;
  sfx::kernels::scatter_kernel<C, NPE, double><<<unsigned((f.nnodes + 255) / 256), 256, 0, s>>>(
      E, f.node_ptr.p, f.node_ent.p, out, f.nnodes, accumulate, int64_t(0), f.nnodes);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("scatter launch: ") + cudaGetErrorString(err));
  return SFX_OK;
}

int scatter_any(const sfx_form_s& f, int C, const double* E, double* out, bool accumulate, cudaStream_t s) {
  if (f.p == 1 && C == 1) return scatter_c<1, 8>(f, E, out, accumulate, s);
  if (f.p == 1 && C == 3) return scatter_c<3, 8>(f, E, out, accumulate, s);
  if (f.p == 2 && C == 1) return scatter_c<1, 27>(f, E, out, accumulate, s);
  if (f.p == 2 && C == 3) return scatter_c<3, 27>(f, E, out, accumulate, s);
  return fail(SFX_ERR_UNSUPPORTED, "field components must be 1 or 3");
}

inline unsigned element_blocks(int64_t ne, int p) {
  const int epw = 32 / ((p + 1) * (p + 1) * (p + 1));
  const int64_t warps = (ne + epw - 1) / epw;
  return unsigned((warps * 32 + 127) / 128);
}

sfx::kernels::MultiArgs<double> args_of(const sfx_mform_s& m, const MultiIntegral& in, const double* const* fields,
                                        const double* dir, double* out_e, double t) {
  const sfx_form_s& f = *m.base;
  sfx::kernels::MultiArgs<double> a{};
  for (size_t k = 0; k < in.args.size(); k++) a.u[k] = fields ? fields[in.args[k]] : nullptr;
  a.dir = dir;
  a.out_e = out_e;
  a.conn = f.conn.p;
  a.geom = f.geom64.p;
  a.state = nullptr;
  a.params = in.params.p;
  a.num_nodes = f.nnodes;
  a.num_elements = f.ne;
  a.t = t;
  return a;
}

// residual (W < 0) or stored derivative with respect to argument W
template <int P, int W>
int launch_param_nh(const sfx_mform_s& m, const MultiIntegral& in, const double* const* fields, double* out_e,
                    double t, cudaStream_t s) {
  using FL = sfx::kernels::FieldList<3, 3, 1, 1>;
  const auto a = args_of(m, in, fields, nullptr, out_e, t);
  sfx::kernels::multi_domain_kernel<P, 3, FL, W, Empty, ParamNeoHookeanMaker>
      <<<element_blocks(m.base->ne, P), 128, 0, s>>>(a, ParamNeoHookeanMaker{}, in.D.p);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("multi-field kernel launch: ") + cudaGetErrorString(err));
  return SFX_OK;
}

template <int P>
int launch_param_nh_w(const sfx_mform_s& m, const MultiIntegral& in, int W, const double* const* fields, double* e,
                      double t, cudaStream_t s) {
  switch (W) {
    case -1: return launch_param_nh<P, -1>(m, in, fields, e, t, s);
    case 0: return launch_param_nh<P, 0>(m, in, fields, e, t, s);
    case 1: return launch_param_nh<P, 1>(m, in, fields, e, t, s);
    case 2: return launch_param_nh<P, 2>(m, in, fields, e, t, s);
    case 3: return launch_param_nh<P, 3>(m, in, fields, e, t, s);
  }
  return fail(SFX_ERR_INVALID, "argument index");
}

int launch_integral(const sfx_mform_s& m, const MultiIntegral& in, int W, const double* const* fields, double* e,
                    double t, cudaStream_t s) {
  if (in.material != SFX_MAT_PARAM_NEOHOOKEAN) return fail(SFX_ERR_UNSUPPORTED, "unknown multi-field material");
  return m.base->p == 1 ? launch_param_nh_w<1>(m, in, W, fields, e, t, s) : launch_param_nh_w<2>(m, in, W, fields, e, t, s);
}

template <int P, int CW, bool TRANSPOSE>
int launch_action(const sfx_mform_s& m, const MultiIntegral& in, const double* dir, double* out_e, cudaStream_t s) {
  const auto a = args_of(m, in, nullptr, dir, out_e, 0.0);
  sfx::kernels::multi_jvp_kernel<P, 3, CW, TRANSPOSE><<<element_blocks(m.base->ne, P), 128, 0, s>>>(a, in.D.p);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(SFX_ERR_CUDA, std::string("multi-field action launch: ") + cudaGetErrorString(err));
  return SFX_OK;
}

int launch_action_any(const sfx_mform_s& m, const MultiIntegral& in, int CW, bool transpose, const double* dir,
                      double* out_e, cudaStream_t s) {
  const int p = m.base->p;
  if (CW == 3) {
    if (p == 1) return transpose ? launch_action<1, 3, true>(m, in, dir, out_e, s) : launch_action<1, 3, false>(m, in, dir, out_e, s);
    return transpose ? launch_action<2, 3, true>(m, in, dir, out_e, s) : launch_action<2, 3, false>(m, in, dir, out_e, s);
  }
  if (CW == 1) {
    if (p == 1) return transpose ? launch_action<1, 1, true>(m, in, dir, out_e, s) : launch_action<1, 1, false>(m, in, dir, out_e, s);
    return transpose ? launch_action<2, 1, true>(m, in, dir, out_e, s) : launch_action<2, 1, false>(m, in, dir, out_e, s);
  }
  return fail(SFX_ERR_UNSUPPORTED, "field components must be 1 or 3");
}

// argument position of form field `field` in integral `in` (-1: not an argument)
int arg_of(const MultiIntegral& in, int field) {
  for (size_t k = 0; k < in.args.size(); k++)
    if (in.args[k] == field) return int(k);
  return -1;
}

int field_count(int material, std::vector<int>* comps) {
  if (material == SFX_MAT_PARAM_NEOHOOKEAN) {
    *comps = {3, 3, 1, 1};  // displacement, acceleration, bulk modulus offset, shear modulus offset
    return 4;
  }
  return fail(SFX_ERR_UNSUPPORTED, "unknown multi-field material");
}

}  // namespace

extern "C" {

int sfx_mform_create(sfx_mesh mesh, int order, int test_components, int num_fields, const int* field_components,
                     sfx_mform* out) {
  if (!mesh || !out || (num_fields > 0 && !field_components)) return fail(SFX_ERR_INVALID, "null argument");
  *out = nullptr;
  if (num_fields < 1 || num_fields > sfx::kernels::kMaxFields) return fail(SFX_ERR_UNSUPPORTED, "1 to 8 fields");
  if (test_components != 3) return fail(SFX_ERR_UNSUPPORTED, "multi-field forms have a 3-component test space");
  for (int i = 0; i < num_fields; i++)
    if (field_components[i] != 1 && field_components[i] != 3) return fail(SFX_ERR_UNSUPPORTED, "field components must be 1 or 3");
  auto* m = new (std::nothrow) sfx_mform_s;
  if (!m) return fail(SFX_ERR_NOMEM, "host allocation failed");
  if (int rc = sfx_form_create(mesh, order, test_components, &m->base)) {
    delete m;
    return rc;
  }
  m->test_components = test_components;
  m->comps.assign(field_components, field_components + num_fields);
  const int cmax = std::max(test_components, *std::max_element(m->comps.begin(), m->comps.end()));
  if (m->E.alloc(size_t(m->base->ne) * size_t(m->base->NPE) * size_t(cmax)) != cudaSuccess) {
    delete m;
    return fail(SFX_ERR_NOMEM, "E-vector scratch");
  }
  *out = m;
  return SFX_OK;
}

int sfx_mform_destroy(sfx_mform form) {
  delete form;
  return SFX_OK;
}

int sfx_mform_num_nodes(sfx_mform form, int64_t* out) {
  if (check(form) || !out) return SFX_ERR_INVALID;
  *out = form->base->nnodes;
  return SFX_OK;
}

int sfx_mform_add_domain_integral(sfx_mform form, int material, const int* depends_on, int num_args,
                                  const double* params, int per_element) {
  if (check(form)) return SFX_ERR_INVALID;
  std::vector<int> want;
  const int n = field_count(material, &want);
  if (n < 0) return n;
  if (num_args != n || !depends_on) return fail(SFX_ERR_INVALID, "the material takes " + std::to_string(n) + " arguments");
  if (!params) return fail(SFX_ERR_INVALID, "null parameters");
  MultiIntegral in;
  in.material = material;
  for (int k = 0; k < n; k++) {
    const int fld = depends_on[k];
    if (fld < 0 || fld >= int(form->comps.size())) return fail(SFX_ERR_INVALID, "DependsOn index out of range");
    if (form->comps[size_t(fld)] != want[size_t(k)])
      return fail(SFX_ERR_INVALID, "argument " + std::to_string(k) + " needs a field of " +
                                       std::to_string(want[size_t(k)]) + " components");
    in.args.push_back(fld);
  }
  const int np = ParamNeoHookeanMaker::nparams;
  const int64_t ne = form->base->ne;
  std::vector<double> prm(size_t(ne) * np);
  for (int64_t e = 0; e < ne; e++)
    for (int k = 0; k < np; k++) prm[size_t(e * np + k)] = per_element ? params[e * np + k] : params[k];
  if (in.params.upload(prm.data(), prm.size()) != cudaSuccess) return fail(SFX_ERR_CUDA, "parameter upload");
  form->integrals.push_back(std::move(in));
  form->lin_field = -1;
  return SFX_OK;
}

int sfx_mform_residual(sfx_mform form, double t, const double* const* fields, double* r, void* stream) {
  if (check(form) || !fields || !r) return fail(SFX_ERR_INVALID, "null argument");
  if (form->integrals.empty()) return fail(SFX_ERR_INVALID, "no integrals");
  for (size_t i = 0; i < form->comps.size(); i++)
    if (!fields[i]) return fail(SFX_ERR_INVALID, "null field");
  auto s = static_cast<cudaStream_t>(stream);
  for (size_t i = 0; i < form->integrals.size(); i++) {
    if (int rc = launch_integral(*form, form->integrals[i], -1, fields, form->E.p, t, s)) return rc;
    if (int rc = scatter_any(*form->base, form->test_components, form->E.p, r, i > 0, s)) return rc;
  }
  return SFX_OK;
}

int sfx_mform_linearize(sfx_mform form, double t, const double* const* fields, int wrt, void* stream) {
  if (check(form) || !fields) return fail(SFX_ERR_INVALID, "null argument");
  if (wrt < 0 || wrt >= int(form->comps.size())) return fail(SFX_ERR_INVALID, "wrt: no such field");
  for (size_t i = 0; i < form->comps.size(); i++)
    if (!fields[i]) return fail(SFX_ERR_INVALID, "null field");
  auto s = static_cast<cudaStream_t>(stream);
  const sfx_form_s& f = *form->base;
  const int cw = form->comps[size_t(wrt)];
  const size_t stride = size_t((int64_t(4 * form->test_components) * 4 * cw * f.NQ + 3) / 4 * 4);
  for (auto& in : form->integrals) {
    in.lin_arg = arg_of(in, wrt);
    if (in.lin_arg < 0) continue;  // this integral does not depend on the field
    if (in.D.n != stride * size_t(f.ne) && in.D.alloc(stride * size_t(f.ne)) != cudaSuccess)
      return fail(SFX_ERR_NOMEM, "derivative storage");
    if (int rc = launch_integral(*form, in, in.lin_arg, fields, nullptr, t, s)) return rc;
  }
  form->lin_field = wrt;
  return SFX_OK;
}

int sfx_mform_jvp(sfx_mform form, int wrt, const double* d_field, double* dr, void* stream) {
  if (check(form) || !d_field || !dr) return fail(SFX_ERR_INVALID, "null argument");
  if (wrt != form->lin_field || wrt < 0) return fail(SFX_ERR_INVALID, "linearise with respect to this field first");
  auto s = static_cast<cudaStream_t>(stream);
  bool first = true;
  for (auto& in : form->integrals) {
    if (in.lin_arg < 0) continue;
    if (int rc = launch_action_any(*form, in, form->comps[size_t(wrt)], false, d_field, form->E.p, s)) return rc;
    if (int rc = scatter_any(*form->base, form->test_components, form->E.p, dr, !first, s)) return rc;
    first = false;
  }
  if (first) SFX_CUDA_TRY(cudaMemsetAsync(dr, 0, sizeof(double) * size_t(form->base->nnodes * form->test_components), s));
  return SFX_OK;
}

int sfx_mform_jvp_transpose(sfx_mform form, int wrt, const double* v, double* out_field, void* stream) {
  if (check(form) || !v || !out_field) return fail(SFX_ERR_INVALID, "null argument");
  if (wrt != form->lin_field || wrt < 0) return fail(SFX_ERR_INVALID, "linearise with respect to this field first");
  auto s = static_cast<cudaStream_t>(stream);
  const int cw = form->comps[size_t(wrt)];
  bool first = true;
  for (auto& in : form->integrals) {
    if (in.lin_arg < 0) continue;
    if (int rc = launch_action_any(*form, in, cw, true, v, form->E.p, s)) return rc;
    if (int rc = scatter_any(*form->base, cw, form->E.p, out_field, !first, s)) return rc;
    first = false;
  }
  if (first) SFX_CUDA_TRY(cudaMemsetAsync(out_field, 0, sizeof(double) * size_t(form->base->nnodes * cw), s));
  return SFX_OK;
}

}  // extern "C"
