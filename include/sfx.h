/*
 * sfx — C ABI of the GB300-native weak-form engine (serac::Functional on
 * hexahedral H1 meshes).  Plain pointers and sizes only; every array argument
 * documented "device" is a CUDA device pointer owned by the caller, every
 * "host" one a host pointer owned by the caller.  `stream` is a cudaStream_t
 * (NULL = the legacy default stream).  Calls are asynchronous on `stream`
 * unless stated otherwise.  All functions return SFX_OK (0) or a negative
 * status; sfx_last_error() describes the last failure on the calling thread.
 *
 * Objects are not thread-safe (like serac::Functional, whose evaluation uses
 * mutable scratch, functional.hpp:723-741): use one form per host thread.
 *
 * Reference interface each entry point replaces (serac, src/serac/...):
 *   sfx_mesh_create_structured_hex  mesh/mesh_utils.cpp:149-153 buildCuboidMesh (+ EnsureNodes, :466)
 *   sfx_form_create                 numerics/functional/functional.hpp:219-273 Functional ctor
 *   sfx_form_create_from_table      the same over an mfem element-dof table (element_restriction.cpp:216-277)
 *   sfx_form_add_domain_integral    numerics/functional/functional.hpp:286-317 AddDomainIntegral
 *   sfx_form_add_boundary_integral  numerics/functional/functional.hpp:328-354 AddBoundaryIntegral
 *   sfx_form_set_shape_displacement numerics/functional/shape_aware_functional.hpp:45-172, 330-560
 *                                   ShapeAwareFunctional (shape displacement as trial 0, held fixed)
 *   sfx_residual                    numerics/functional/functional.hpp:502-513 operator()(t, u)
 *   sfx_linearize                   numerics/functional/functional.hpp:481-489 operator()(t, differentiate_wrt(u))
 *   sfx_jvp / sfx_jvp_f32           numerics/functional/functional.hpp:556-566 Gradient::Mult / operator()
 *   sfx_jvp_host                    the same Gradient::Mult on host-resident mfem::Vectors (mfem moves them to
 *                                   and from the device around the action)
 *   sfx_jvp_element(_f32)           numerics/functional/integral.hpp:93-103 Integral::GradientMult
 *   sfx_jvp_transpose(_f32)         physics/solid_mechanics.hpp:1343-1501 (the adjoint solves' transposed
 *                                   Jacobian, formed there as the transpose of assemble(Gradient&))
 *   sfx_shape_vjp                   physics/solid_mechanics.hpp:1421-1431, 1495-1503 (assemble(dR/dshape)
 *                                   followed by MultTranspose(adjoint))
 *   sfx_qoi_*                       numerics/functional/functional_qoi.inl:58-528 Functional<double(trials...)>:
 *                                   AddDomainIntegral :159-189, AddBoundaryIntegral :201-228, operator() :379-392,
 *                                   Gradient::operator() :420, Gradient::assemble :422-475
 *   sfx_csr_* / sfx_assemble_csr    numerics/functional/functional.hpp:569-667 assemble(Gradient&)
 *   sfx_set_param_field             physics/base_physics.hpp:300 BasePhysics::setParameter (a parameter
 *                                   field of the physics module), as per-element values
 *   sfx_update_qdata                numerics/functional/functional.hpp:523 updateQdata(bool)
 *   sfx_set_qdata / sfx_get_qdata   numerics/functional/quadrature_data.hpp:111-144 QuadratureData<T>
 */
#ifndef SFX_H
#define SFX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFX_OK 0
#define SFX_ERR_INVALID (-1)     /* bad argument or call order */
#define SFX_ERR_CUDA (-2)        /* a CUDA call failed */
#define SFX_ERR_NONFINITE (-3)   /* a non-finite value was detected */
#define SFX_ERR_TIMEOUT (-4)     /* a bounded device-side wait expired */
#define SFX_ERR_UNSUPPORTED (-5) /* order / material / size not built */
#define SFX_ERR_NOMEM (-6)       /* device allocation failed */

/* Domain materials (q-functions instantiated in this library). Parameters per
 * element, in this order:
 *   SFX_MAT_HEAT            {k, f}            steady conduction, source f (heat_transfer.hpp:381-400, 488-505)
 *   SFX_MAT_NEOHOOKEAN      {K, G}            MaterialStressFunctor<NeoHookean> (solid_material.hpp:98-127)
 *   SFX_MAT_J2              {E, nu, sigma_y, H}  J2SmallStrain<LinearHardening>, small strain (solid_material.hpp:199-258)
 *   SFX_MAT_THERMAL_TEST    {}                linear scalar model, all derivative blocks populated
 *   SFX_MAT_ELASTIC_TEST    {}                linear vector model, all derivative blocks populated
 *   SFX_MAT_NONLINEAR_HEAT  {k0, beta, f}     k(u) = k0 (1 + beta u^2)
 */
#define SFX_MAT_HEAT 0
#define SFX_MAT_NEOHOOKEAN 1
#define SFX_MAT_J2 2
#define SFX_MAT_THERMAL_TEST 3
#define SFX_MAT_ELASTIC_TEST 4
#define SFX_MAT_NONLINEAR_HEAT 5
/* Multi-field material (sfx_mform_add_domain_integral), per-element
 * parameters {density, K0, G0}, arguments (displacement 3, acceleration 3,
 * bulk modulus offset 1, shear modulus offset 1):
 *   SFX_MAT_PARAM_NEOHOOKEAN  {density a, P(grad u; K0 + dK, G0 + dG)}
 *   (ParameterizedNeoHookeanSolid, parameterized_solid_material.hpp:68-110, in
 *   SolidMechanics' material integrand with acceleration, solid_mechanics.hpp:809-850) */
#define SFX_MAT_PARAM_NEOHOOKEAN 16

/* Boundary materials: SFX_BMAT_HEAT_FLUX {q0, q1, alpha}: -(q0 + q1 x + alpha u);
 * SFX_BMAT_TRACTION {t0[3], t1[3]}: -(t0 + t1 x); SFX_BMAT_PRESSURE {p}:
 * p n(deformed) / |n(reference)| (solid_mechanics.hpp:1029-1099). */
#define SFX_BMAT_HEAT_FLUX 0
#define SFX_BMAT_TRACTION 1
#define SFX_BMAT_PRESSURE 2

/* Boundary sides of the structured box, as a bit mask (bit s-1 for side s):
 * 1: z=0, 2: y=0, 3: x=1, 4: y=1, 5: x=0, 6: z=1. */

typedef struct sfx_mesh_s* sfx_mesh;
typedef struct sfx_form_s* sfx_form;
typedef struct sfx_mform_s* sfx_mform;

const char* sfx_last_error(void);
int sfx_version(void);

/* Structured nx x ny x nz hexahedral mesh with trilinear geometry.
 * vertices: host, (nx+1)(ny+1)(nz+1) x 3 doubles, vertex (i,j,k) at row
 * i + (nx+1)(j + (ny+1)k).  The mesh copies the coordinates. */
int sfx_mesh_create_structured_hex(int nx, int ny, int nz, const double* vertices, sfx_mesh* out);
int sfx_mesh_destroy(sfx_mesh mesh);
int sfx_mesh_num_elements(sfx_mesh mesh, int64_t* out);

/* Functional<H1<order, components>(H1<order, components)> on `mesh`
 * (order 1 or 2; components 1 or 3).  Q = order + 1 Gauss points per
 * direction.  Global numbering: H1 node (I, J, K) of the
 * (order nx + 1)(order ny + 1)(order nz + 1) grid is I + Nx (J + Ny K); the
 * vector layout is byNODES: vdof = component * num_nodes + node. */
int sfx_form_create(sfx_mesh mesh, int order, int components, sfx_form* out);

/* The same for any conforming hexahedral mesh, from an imported element-dof
 * table (the one mfem's ParFiniteElementSpace holds for serac's H1 spaces,
 * element_restriction.cpp:216-277, after its native -> lexicographic
 * permutation): elem_nodes (host, num_elements x (order+1)^3 int32) gives
 * each element's scalar node ids in lexicographic local order (x fastest),
 * the caller's own numbering in [0, num_nodes) (vdof = component *
 * num_nodes + node); elem_vertices (host, num_elements x 8 x 3 doubles) the
 * element's corner coordinates in lexicographic corner order (trilinear
 * geometry, positively oriented: an element whose Jacobian at its centre
 * is not positive, as a wrong node or corner permutation gives, is rejected
 * with SFX_ERR_INVALID).  Only the centre is checked: an element that is
 * valid there but has det J <= 0 at some quadrature point (inverted near a
 * corner) is accepted, as serac accepts it, and gives wrong or non-finite
 * results; such meshes are the caller's to reject.  Every operator of this header works on
 * such a form; boundaries are given as face lists
 * (sfx_form_add_boundary_integral_faces), the CSR graph is the union of the
 * element node sets per node (columns sorted), and results follow the
 * caller's numbering.  For order <= 2 every edge and face carries at most
 * one node, so no orientation data is needed. */
int sfx_form_create_from_table(int order, int components, int64_t num_elements, int64_t num_nodes,
                               const int32_t* elem_nodes, const double* elem_vertices, sfx_form* out);
int sfx_form_destroy(sfx_form form);
int sfx_form_num_dofs(sfx_form form, int64_t* out);

/* params: host; if per_element != 0, num_elements x nparams values, else
 * nparams values used for every element.  At most one domain integral per
 * form in this version. */
int sfx_form_add_domain_integral(sfx_form form, int material, const double* params, int per_element);

/* Replace the material parameters of domain integral `integral` (0-based, in
 * the order added; params: host, as for sfx_form_add_domain_integral) without
 * rebuilding the form: a parameter field updated between evaluations, e.g. in
 * a design loop.  Synchronous: it first waits for all work queued on the
 * device (every stream), so no evaluation in flight sees a mix of old and
 * new parameters; the form must be linearised again. */
int sfx_set_param_field(sfx_form form, int integral, const double* params, int per_element);

/* Boundary integral over the faces of the sides in side_mask; params: host. */
int sfx_form_add_boundary_integral(sfx_form form, int bmaterial, int side_mask, const double* params);
/* The same over an explicit face list (host arrays of num_faces entries):
 * face_elem[k] an element, face_side[k] its local side (1: zeta=0, 2: eta=0,
 * 3: xi=1, 4: eta=1, 5: xi=0, 6: zeta=1 in the element's lexicographic frame),
 * like mfem's boundary elements of an attribute. */
int sfx_form_add_boundary_integral_faces(sfx_form form, int bmaterial, int64_t num_faces, const int32_t* face_elem,
                                         const int32_t* face_side, const double* params);

/* Shape displacement p (device, 3 * num_nodes doubles, byNODES on the form's
 * node grid; NULL = none): every integral of the form is evaluated on the
 * configuration x = X + p as serac's ShapeAwareFunctional does — trial
 * gradients du/dX (I + dp/dX)^-1, domain outputs scaled by det(I + dp/dX)
 * with the flux mapped by (I + dp/dX)^-T, boundary weights by the area ratio,
 * and the q-function position argument X + p.  The value is copied; the form
 * must be linearised again afterwards. */
int sfx_form_set_shape_displacement(sfx_form form, const double* shape, void* stream);

/* dr = dR/dp (t, u; p) dshape: the derivative of the residual with respect to
 * the shape displacement p set on the form (zero when none is set), applied to
 * dshape (device, 3 * num_nodes doubles) — ShapeAwareFunctional differentiated
 * with respect to its argument 0 (shape_aware_functional.hpp:537-541), for
 * its domain and boundary integrals. */
int sfx_shape_jvp(sfx_form form, double t, const double* u, const double* dshape, double* dr, void* stream);

/* out = (dR/dp (t, u; p))^T lam (device, 3 * num_nodes doubles): the shape
 * sensitivity of an adjoint problem, which serac forms by assembling dR/dp
 * and applying its transpose (SolidMechanics::computeTimestepShapeSensitivity,
 * solid_mechanics.hpp:1421-1431; computeDualShapeSensitivity, :1495-1503),
 * matrix-free over the domain and boundary integrals. */
int sfx_shape_vjp(sfx_form form, double t, const double* u, const double* lam, double* out, void* stream);

/* r = R(t, u) (device, num_dofs doubles each).  When sfx_update_qdata(form, 1)
 * is in effect, quadrature-point state is committed by this call. */
int sfx_residual(sfx_form form, double t, const double* u, double* r, void* stream);

/* Record the linearisation point (t, u) for sfx_jvp / sfx_jvp_f32 /
 * sfx_assemble_csr; also writes R(t, u) to r when r != NULL.  The form keeps
 * its own copy of u (FP64 and FP32). */
int sfx_linearize(sfx_form form, double t, const double* u, double* r, void* stream);

/* How sfx_jvp applies the linearisation:
 *   SFX_JVP_STORED_TANGENT (default): sfx_linearize evaluates the q-function
 *     derivative at every quadrature point once and stores it (FP64 and FP32
 *     copies, serac's own scheme: domain_integral_kernels.hpp:209-214, 277-304);
 *     each Jacobian action then only interpolates du, applies it and integrates.
 *   SFX_JVP_RECOMPUTE: nothing is stored; every Jacobian action re-evaluates
 *     the q-function on directional dual numbers (less memory, more FP64 work). */
#define SFX_JVP_STORED_TANGENT 0
#define SFX_JVP_RECOMPUTE 1
int sfx_form_set_jvp_mode(sfx_form form, int mode);

/* Storage of the tangent copy that the FP32 action streams (the inner
 * Krylov operator of the mixed-precision solver): SFX_TANGENT_F32 (default)
 * or SFX_TANGENT_F16 (half the bytes, about 3 significant digits per entry,
 * FP32 accumulation; order 2).  The FP64 tangent is unaffected.  Takes effect
 * at the next sfx_linearize. */
#define SFX_TANGENT_F32 0
#define SFX_TANGENT_F16 1
int sfx_form_set_tangent_storage(sfx_form form, int storage);

/* dr = dR/du(t_lin, u_lin) du, in FP64, and in FP32 (FP32 accumulation). */
int sfx_jvp(sfx_form form, const double* du, double* dr, void* stream);
int sfx_jvp_f32(sfx_form form, const float* du, float* dr, void* stream);

/* dr = dR/du(t_lin, u_lin) du in FP64 with du and dr in HOST memory (ndofs
 * doubles each; page-locked memory lets the copies overlap the kernels).  On
 * a structured mesh with one domain integral, no boundary integral and the
 * stored tangent, the copies in, the element kernels, the scatter and the
 * copies out are pipelined over (up to 8) slabs of element layers in z, on
 * two internal copy streams and `stream`: slab k's elements need the node
 * planes up to the slab's top, and the node planes below it are complete
 * once slab k is done.  Other forms copy in, run sfx_jvp and copy out.  The
 * result is bitwise that of sfx_jvp.  Blocks until dr is written; two
 * device vectors of ndofs doubles are allocated on the first call and kept
 * with the form. */
int sfx_jvp_host(sfx_form form, const double* du, double* dr, void* stream);

/* Element-level Jacobian action before the scatter-add (Integral::GradientMult,
 * integral.hpp:93-103): dE[e][component][node] (device, num_elements *
 * components * (order+1)^3 doubles) for the domain integral. */
int sfx_jvp_element(sfx_form form, const double* du, double* dE, void* stream);
/* The same in FP32 on the FP32 stored tangent (dE: num_elements * c * (p+1)^3 floats). */
int sfx_jvp_element_f32(sfx_form form, const float* du, float* dE, void* stream);

/* dr = dR/du(t_lin, u_lin)^T v: the transposed Jacobian action for adjoint
 * problems (serac assembles the Jacobian and transposes it,
 * solid_mechanics.hpp:1343-1501), matrix-free: the domain part applies the
 * stored tangent transposed (needs SFX_JVP_STORED_TANGENT), boundary
 * integrals re-linearise their q-functions per face point.  FP64, and FP32
 * on the FP32 tangent. */
int sfx_jvp_transpose(sfx_form form, const double* v, double* dr, void* stream);
int sfx_jvp_transpose_f32(sfx_form form, const float* v, float* dr, void* stream);

/* Self-test of the device-side bounded waits (the mbarrier waits of the
 * bulk-copy kernels): one block waits, for at most `polls` polls, on a barrier
 * that nothing completes; returns SFX_ERR_TIMEOUT when the bound worked, as it
 * must, and leaves the context usable. */
int sfx_selftest_bounded_wait(unsigned polls);
/* Self-test of the tensor-core (tcgen05) path used by the learned
 * preconditioner's convolutions: D = A B^T on one 128-row tile, A [128][K] and
 * B [N][K] BF16 row-major, D [128][N] FP32 (device pointers), N in
 * {16, 32, 48, 64, 128}, K a multiple of 16 up to 256.  No counterpart in
 * serac. */
int sfx_selftest_umma_tile(const void* A, const void* B, int N, int K, float* D);

/* Sparsity of dR/du: every (test vdof, trial vdof) pair of every element,
 * rows sorted, columns sorted within a row (dof_numbering.hpp:290-351).
 * row_ptr: device, num_dofs + 1 int64; col: device, nnz int32. */
int sfx_csr_nnz(sfx_form form, int64_t* nnz);
int sfx_csr_graph(sfx_form form, int64_t* row_ptr, int32_t* col, void* stream);
/* values: device, nnz doubles, dR/du at the linearisation point. */
int sfx_assemble_csr(sfx_form form, double* values, void* stream);

/* Diagonal of dR/du at the linearisation point (device, num_dofs doubles). */
int sfx_assemble_diagonal(sfx_form form, double* diag, void* stream);

/* Device-side layout of a form, for the header-only C++ front-end
 * (include/sfx/functional.hpp) that instantiates the element kernels for
 * user q-functions in the caller's translation unit.  It corresponds to the
 * members serac's Functional keeps for its integrals (element restriction
 * tables, geometric factors and E-vector scratch: functional.hpp:723-741,
 * geometric_factors.hpp).  Pointers stay valid until the form is destroyed;
 * row_ptr is NULL until the CSR graph has been built (sfx_csr_nnz). */
typedef struct {
  int order, components;
  int64_t num_elements, num_nodes, num_dofs;
  const int32_t* conn;     /* [e][(order+1)^3] node ids */
  const int32_t* node_ptr; /* [num_nodes + 1] node -> (element, local) entries */
  const int32_t* node_ent; /* e * (order+1)^3 + local, element order */
  const double* geom;      /* 22 x num_elements (order+1)^3 point factors (sfx/kernels.cuh GEOM_STRIDE) */
  const float* geom_f32;
  double* evector;         /* scratch [e][component][node] */
  float* evector_f32;
  const int64_t* row_ptr;  /* CSR rows (num_dofs + 1) or NULL */
  int nx, ny, nz;          /* structured forms: elements per direction (0 for table forms) */
  int general;             /* 1 for forms built by sfx_form_create_from_table */
  const int64_t* graph_ptr; /* table forms: sorted scalar adjacency [num_nodes + 1] (NULL until the CSR graph is built) */
  const int32_t* graph_col;
  const double* elem_vertices; /* [e][3][8] reference corner coordinates */
  const double* shape;     /* shape displacement [3][num_nodes], NULL when none is set */
} sfx_form_layout;
int sfx_form_get_layout(sfx_form form, sfx_form_layout* out);

/* Face sets for boundary integrals whose q-functions the caller evaluates in
 * its own kernels (the C++ front-end's AddBoundaryIntegral with user
 * q-functions, functional.hpp:328-354): the faces of the sides in side_mask
 * (1: z=0, 2: y=0, 3: x=1, 4: y=1, 5: x=0, 6: z=1), their geometric factors
 * (shape-displaced with the form) and the compact face-node map of the
 * deterministic face scatter. */
typedef struct {
  int64_t num_faces;
  int nodes_per_face;       /* (order+1)^2, also the points per face */
  const int32_t* fconn;     /* [face][nodes_per_face] node ids, outward (s, t) order */
  const double* fgeom;      /* 10 x num_faces * nodes_per_face point factors (sfx/boundary.cuh FGEOM_STRIDE) */
  int64_t num_face_nodes;   /* distinct nodes of the set */
  const int32_t* node_ptr;  /* [num_face_nodes + 1] entries per distinct node */
  const int32_t* node_ids;  /* global node of each distinct node */
  const int32_t* node_ent;  /* face * nodes_per_face + local, face order */
  const double* face_vertices; /* [face][3][4] reference corner coordinates, outward (s, t) order */
} sfx_face_layout;
int sfx_form_add_face_set(sfx_form form, int side_mask, int* face_set);
int sfx_form_add_face_set_faces(sfx_form form, int64_t num_faces, const int32_t* face_elem, const int32_t* face_side,
                                int* face_set);
int sfx_form_get_face_layout(sfx_form form, int face_set, sfx_face_layout* out);

/* out = (accumulate ? out : 0) + scatter-add of the E-vector E [e][component][node]
 * (ElementRestriction::ScatterAdd, element_restriction.cpp:456-467), node-owner
 * order, deterministic. */
int sfx_scatter_add(sfx_form form, const double* E, double* out, int accumulate, void* stream);
int sfx_scatter_add_f32(sfx_form form, const float* E, float* out, int accumulate, void* stream);

/* Residual of a structured mesh that allocates nothing (no counterpart in
 * serac).  For callers that cannot allocate device memory at call time or at
 * all (a memory manager owns every device allocation, or the device footprint
 * must not grow after start-up): the caller passes the vertex coordinates
 * (device, (nx+1)(ny+1)(nz+1) x 3 doubles), the field u and the output r
 * (device, num_dofs doubles each) and the material parameters (host, as for
 * sfx_form_add_domain_integral, uniform); the connectivity and the geometry
 * are derived from the grid inside the kernels, and the element-residual
 * scratch is a fixed 32 MiB device array inside this library (held on every
 * device that loads the library until exit), so num_elements * components *
 * (order+1)^3 must not exceed 4,194,304 (SFX_ERR_UNSUPPORTED otherwise).
 * Materials: SFX_MAT_HEAT, SFX_MAT_NEOHOOKEAN; order 1 or 2.  The first call
 * on a device looks up the scratch array's device address (make it before
 * any stream capture); the address is cached per device and context, so a
 * device reset or a new context is followed by a fresh lookup.  Every call on a device shares the scratch array:
 * calls that overlap on that device race and must be serialised by the
 * caller.  Results equal sfx_residual's for the same mesh and material. */
int sfx_residual_structured_noalloc(int nx, int ny, int nz, int order, int material, const double* params,
                                    const double* vertices, const double* u, double* r, double t, void* stream);

/* Quantities of interest: Functional<double(H1<order, components>)>
 * (functional_qoi.inl:58-528).  A QoI form integrates scalar integrands over
 * the domain and / or box sides; its value, its directional derivative and
 * its gradient dQ/du are device results.  Integrand kinds (parameters, host,
 * in this order; q is integrated with det(J) w on the domain and
 * |dX/ds x dX/dt| w on faces):
 *   SFX_QOI_MEASURE            {}        1: volume / area
 *   SFX_QOI_POSITION           {a[3]}    a . X
 *   SFX_QOI_FIELD              {w[c]}    w . u
 *   SFX_QOI_NEOHOOKEAN_ENERGY  {K, G}    stored energy of SFX_MAT_NEOHOOKEAN (domain, c = 3);
 *                                        its gradient is that material's residual
 *   SFX_QOI_NORMAL_FIELD       {}        u . n, n the outward unit normal (faces, c = 3)
 *   SFX_QOI_POLY_TEST          {}        nonlinear test integrand (sfx/qoi.cuh)
 * A QoI form is created by sfx_qoi_create (destroyed by sfx_form_destroy) and
 * takes sfx_form_set_shape_displacement; the residual entry points reject it. */
#define SFX_QOI_MEASURE 0
#define SFX_QOI_POSITION 1
#define SFX_QOI_FIELD 2
#define SFX_QOI_NEOHOOKEAN_ENERGY 3
#define SFX_QOI_NORMAL_FIELD 4
#define SFX_QOI_POLY_TEST 5
int sfx_qoi_create(sfx_mesh mesh, int order, int components, sfx_form* out);
int sfx_qoi_add_domain_integral(sfx_form qoi, int kind, const double* params);
int sfx_qoi_add_boundary_integral(sfx_form qoi, int kind, int side_mask, const double* params);
int sfx_qoi_create_from_table(int order, int components, int64_t num_elements, int64_t num_nodes,
                              const int32_t* elem_nodes, const double* elem_vertices, sfx_form* out);
int sfx_qoi_add_boundary_integral_faces(sfx_form qoi, int kind, int64_t num_faces, const int32_t* face_elem,
                                        const int32_t* face_side, const double* params);
/* value: device, one double = Q(t, u) */
int sfx_qoi_evaluate(sfx_form qoi, double t, const double* u, double* value, void* stream);
/* grad: device, num_dofs doubles = dQ/du (t, u); value (device, one double)
 * receives Q(t, u) unless NULL */
int sfx_qoi_gradient(sfx_form qoi, double t, const double* u, double* value, double* grad, void* stream);
/* out: device, one double = dQ/du (t, u) du */
int sfx_qoi_action(sfx_form qoi, double t, const double* u, const double* du, double* out, void* stream);
/* out: device, 3 * num_nodes doubles = dQ/dp (t, u; p), the partial derivative
 * of the QoI with respect to the shape displacement (the shape-aware QoI
 * differentiated with respect to its shape argument, shape_aware_functional.hpp) */
int sfx_qoi_shape_gradient(sfx_form qoi, double t, const double* u, double* out, void* stream);

/* Quadrature-point state (J2: 10 doubles per point: plastic strain 3x3
 * row-major, accumulated plastic strain), host arrays
 * [element][point][10].  flag: commit state on the next residual calls. */
int sfx_update_qdata(sfx_form form, int flag);
int sfx_qdata_size(sfx_form form, int64_t* num_doubles);
int sfx_set_qdata(sfx_form form, const double* host_state);
int sfx_get_qdata(sfx_form form, double* host_state);

/* Multi-field forms: Functional<test(trial_0, ..., trial_{n-1})>
 * (functional.hpp:189-317), the form SolidMechanics builds as
 * test(displacement, acceleration, parameters...) (solid_mechanics.hpp:243).
 * Every field is H1 of the form's order on the mesh's node grid (an H1 field
 * of lower order is represented exactly by its values there), byNODES
 * ([component][node]); field_components[i] is 1 or 3; the test space has 3
 * components.  Fields are passed as a host array of num_fields device
 * pointers. */
int sfx_mform_create(sfx_mesh mesh, int order, int test_components, int num_fields, const int* field_components,
                     sfx_mform* out);
int sfx_mform_destroy(sfx_mform form);
int sfx_mform_num_nodes(sfx_mform form, int64_t* out);
/* AddDomainIntegral(Dimension<3>, DependsOn<depends_on...>, material): the
 * material's arguments, in order, are the form fields depends_on[0..num_args);
 * params: host, as for sfx_form_add_domain_integral. */
int sfx_mform_add_domain_integral(sfx_mform form, int material, const int* depends_on, int num_args,
                                  const double* params, int per_element);
/* r = R(t, fields...) (test space, 3 x num_nodes). */
int sfx_mform_residual(sfx_mform form, double t, const double* const* fields, double* r, void* stream);
/* operator()(t, ..., differentiate_wrt(field wrt), ...): stores, per
 * quadrature point, the derivative of every integral that depends on field
 * `wrt` with respect to it (an integral that does not contributes zero). */
int sfx_mform_linearize(sfx_mform form, double t, const double* const* fields, int wrt, void* stream);
/* dr = dR/d(field wrt) d_field (Gradient::Mult for that argument); wrt must
 * be the field of the last sfx_mform_linearize. */
int sfx_mform_jvp(sfx_mform form, int wrt, const double* d_field, double* dr, void* stream);
/* out_field = (dR/d(field wrt))^T v: the test-space vector v mapped onto the
 * field (what a sensitivity with respect to a parameter field needs). */
int sfx_mform_jvp_transpose(sfx_mform form, int wrt, const double* v, double* out_field, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SFX_H */
