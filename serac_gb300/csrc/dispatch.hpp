// Entry points of the per-material kernel instantiations.
#pragma once

#include <cuda_runtime.h>

#include "form.hpp"

namespace sfx_impl {

int material_info(int material, int* components, int* nparams, int* state_doubles);

// mode: 0 residual, 1 residual committing state, 2 Jacobian action (FP64)
int launch_domain(const sfx_form_s& f, const DomainIntegral& di, int mode, const double* u, const double* du,
                  double* E, double t, cudaStream_t s);
// element matrices K[e - e0][trial][test] of elements [e0, e1) at the
// linearisation point, or (diag_only) their diagonals as an E-vector over all elements
int launch_element_matrix(const sfx_form_s& f, const DomainIntegral& di, bool diag_only, double* out, int64_t e0,
                          int64_t e1, cudaStream_t s);
// scatter-add of an E-vector [e][c][node] into an L-vector
int scatter_evector(const sfx_form_s& f, const double* E, double* out, bool accumulate, cudaStream_t s);
/// out[c * N + n] = the element sum of E for the nodes [n0, n1) only (no accumulate)
int scatter_evector_range(const sfx_form_s& f, const double* E, double* out, int64_t n0, int64_t n1,
                          cudaStream_t s);

// stored-tangent path: linearise (store D, optionally element residuals) and apply D
int launch_linearize(const sfx_form_s& f, DomainIntegral& di, double* res_e, cudaStream_t s);
int launch_jvp_stored(const sfx_form_s& f, const DomainIntegral& di, const double* du, double* E, cudaStream_t s);
/// the FP64 stored-tangent action over the elements [e0, e1) only (E indexed globally)
int launch_jvp_stored_range(const sfx_form_s& f, const DomainIntegral& di, const double* du, double* E, int64_t e0,
                            int64_t e1, cudaStream_t s);
// boundary integrals: add face contributions to out (mode 0 residual at u, 2 action on du)
int launch_boundary(const sfx_form_s& f, int mode, const double* u, const double* du, double* out, double t,
                    cudaStream_t s);
int launch_boundary_jvp_f32(const sfx_form_s& f, const float* u, const float* du, float* out, double t,
                            cudaStream_t s);
// face element matrices at the linearisation point added into CSR values and/or a diagonal
int assemble_boundary(sfx_form_s& f, double* values, double* diag, cudaStream_t s);
// derivative of the domain residual with respect to the shape displacement, applied to dshape
int launch_shape_jvp(const sfx_form_s& f, const DomainIntegral& di, const double* u, const double* dshape, double* E,
                     double t, cudaStream_t s);
// out += derivative of the boundary residual with respect to the shape displacement, applied to dshape
int launch_boundary_shape_jvp(const sfx_form_s& f, const double* u, const double* dshape, double* out, double t,
                              cudaStream_t s);
// shape sensitivities: (dR/dp)^T lam of the domain integral as an E-vector
// [e][3][node]; the boundary integrals' part added into out (3 x num_nodes)
int launch_shape_vjp(const sfx_form_s& f, const DomainIntegral& di, const double* u, const double* lam, double* E,
                     double t, cudaStream_t s);
int launch_boundary_shape_vjp(const sfx_form_s& f, const double* u, const double* lam, double* out, double t,
                              cudaStream_t s);
// scatter-add of a 3-component E-vector [e][3][node] (shape space)
int scatter_evector3(const sfx_form_s& f, const double* E, double* out, bool accumulate, cudaStream_t s);
// E-vector scratch of the shape-space kernels (elements and the largest face set)
int ensure_shape_scratch(sfx_form_s& f);
// geometric factors (reference or shape-displaced configuration)
int compute_face_geometry(sfx_form_s& f, BoundaryIntegral& bi, cudaStream_t s);
int compute_geometry(sfx_form_s& f, cudaStream_t s);
// faces of the box sides in side_mask: tables, vertex coordinates, factors, scratch
int build_faces(sfx_form_s* form, int side_mask, BoundaryIntegral& bi);
// faces given as (element, local side 1..6) pairs, in the element's own frame
int build_faces_list(sfx_form_s* form, int64_t n, const int32_t* face_elem, const int32_t* face_side,
                     BoundaryIntegral& bi);

// transposed Jacobian actions: domain from the stored tangent (E-vector),
// boundary added into out
int launch_jvp_transpose(const sfx_form_s& f, const DomainIntegral& di, const double* v, double* E, cudaStream_t s);
int launch_jvp_transpose_f32(const sfx_form_s& f, const DomainIntegral& di, const float* v, float* E,
                             cudaStream_t s);
int launch_boundary_transpose(const sfx_form_s& f, const double* v, double* out, cudaStream_t s);
int launch_boundary_transpose_f32(const sfx_form_s& f, const float* v, float* out, cudaStream_t s);

// diagonal of the element Jacobians from the stored tangent (E-vector)
int launch_diag_from_tangent(const sfx_form_s& f, const DomainIntegral& di, double* E, cudaStream_t s);
int launch_jvp_stored_f32(const sfx_form_s& f, const DomainIntegral& di, const float* du, float* E, cudaStream_t s);

int launch_domain_jvp_f32(const sfx_form_s& f, const DomainIntegral& di, const float* u, const float* du, float* E,
                          double t, cudaStream_t s);

}  // namespace sfx_impl
