/*
 * sfx — device-resident Newton-Krylov solver over an sfx form (C ABI).
 *
 * Replaces serac's solver stack for the quasi-static physics solve
 * (src/serac/numerics/equation_solver.cpp and solver_config.hpp):
 *   sfx_solver_default_options  solver_config.hpp:342-400 LinearSolverOptions / NonlinearSolverOptions
 *   sfx_solver_create           equation_solver.cpp:820-950 buildNonlinearSolver / buildLinearSolverAndPreconditioner
 *   sfx_solver_set_essential    physics/boundary_conditions/boundary_condition_manager.hpp:91 (essential dofs)
 *   sfx_solver_solve            equation_solver.cpp:79-200 NewtonSolver::Mult (quasiStaticSolve, solid_mechanics.hpp:1620-1630)
 *   sfx_solver_warm_start       SolidMechanics::warmStartDisplacement (solid_mechanics.hpp:1727-1770)
 *   sfx_solver_solve_linear     one linearised solve with the essential rows eliminated
 *   sfx_solver_solve_adjoint    the adjoint solve J^T lambda = dQ/du of SolidMechanics::reverseAdjointTimestep
 *                               (solid_mechanics.hpp:1343-1501), matrix-free (sfx_jvp_transpose)
 * The Chebyshev, flexible-GMRES and mixed-precision options have no
 * counterpart in serac (its LinearSolver enum is CG / GMRES / direct / PETSc).
 */
#ifndef SFX_SOLVER_H
#define SFX_SOLVER_H

#include <stdint.h>

#include "sfx.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SFX_ERR_NOT_CONVERGED (-7)

#define SFX_KRYLOV_GMRES 0  /* restarted GMRES(restart), right preconditioned */
#define SFX_KRYLOV_CG 1     /* conjugate gradients (symmetric positive definite) */
#define SFX_KRYLOV_FGMRES 2 /* flexible GMRES (preconditioner may vary per step) */

#define SFX_PREC_NONE 0
#define SFX_PREC_JACOBI 1
#define SFX_PREC_JACOBI_CHEBYSHEV 2
/* Learned multilevel network (include/sfx_learned.h) as the first stage of
 * each outer flexible-GMRES preconditioner application: z = a NN(v) with a
 * minimising |v - a J NN(v)|, then, on what it leaves of v, the inner FP32
 * GMRES(inner_iterations) with FP32 Jacobi-Chebyshev (mixed_precision = 1)
 * or one FP32 Jacobi-Chebyshev application (mixed_precision = 0, see
 * learned_cycle).  A network step that takes less than 1 % off the residual
 * norm is skipped (counted in sfx_solver_stats.learned_fallbacks), leaving the
 * method without the network. */
#define SFX_PREC_LEARNED 3

typedef struct {
  int max_newton_iterations; /* 20 */
  double newton_rel_tol;     /* 1e-8: ||r|| <= rel ||r0|| */
  double newton_abs_tol;     /* 1e-12 */
  int krylov;                /* SFX_KRYLOV_* (GMRES) */
  int restart;               /* 50 */
  int max_krylov_iterations; /* 300 per linear solve */
  double krylov_rel_tol;     /* 1e-8 */
  double krylov_abs_tol;     /* 1e-12 */
  int precond;               /* SFX_PREC_* (Jacobi-Chebyshev) */
  int chebyshev_degree;      /* 3: Chebyshev polynomial degree (degree-1 Jacobian actions) */
  double chebyshev_ratio;    /* 30: interval [lmax / ratio, 1.05 lmax] of D^-1 J */
  int eigen_iterations;      /* 20: Lanczos steps of the lmax estimate per linearisation (largest Ritz value
                                plus its residual bound, from a pseudo-random start vector) */
  int mixed_precision;       /* 1: FP64 flexible GMRES outside, FP32 GMRES + FP32 Jacobi-Chebyshev inside */
  int inner_iterations;      /* 40: FP32 inner GMRES steps per outer step (at most 256; one cycle, run as one CUDA graph) */
  double inner_rel_tol;      /* 1e-3 */
  int print_level;           /* 0 */
  int learned_cycle;         /* 1: SFX_PREC_LEARNED without mixed precision: 1 Chebyshev, network on
                                the smoothed residual, Chebyshev (two-level cycle); 0 network, Chebyshev */
  int inner_chebyshev_degree; /* 0: degree of the FP32 Chebyshev inside the mixed-precision solve
                                 (0: chebyshev_degree) */
  int learned_max_rejections; /* 3: after this many network steps in a row are skipped (each taking less
                                 than 1 % off the residual), the rest of the linear solve runs without the
                                 network (counted in learned_skipped); 0: always try the network */
} sfx_solver_options;

typedef struct {
  int newton_iterations;
  int krylov_iterations; /* outer (FP64) Krylov steps over the whole solve */
  int inner_iterations;  /* inner FP32 Krylov steps (mixed precision) */
  int converged;
  double initial_residual;
  double final_residual;
  double last_krylov_rel;
  int learned_applications; /* network preconditioner applications */
  int learned_fallbacks;    /* of which fell back to Jacobi-Chebyshev */
  double lmax_estimate;     /* the last estimate of the largest eigenvalue of D^-1 J (Chebyshev interval) */
  int learned_skipped;      /* preconditioner applications that did not try the network (learned_max_rejections) */
} sfx_solver_stats;

typedef struct sfx_solver_s* sfx_solver;

int sfx_solver_default_options(sfx_solver_options* opt);
int sfx_solver_create(sfx_form form, const sfx_solver_options* opt, sfx_solver* out);
int sfx_solver_destroy(sfx_solver solver);
/* Essential (Dirichlet) vdofs, host array; their values are taken from u. */
int sfx_solver_set_essential(sfx_solver solver, const int64_t* dofs, int64_t n);
/* Newton solve of R(t, u) = 0 in place (u: device, num_dofs doubles). */
int sfx_solver_solve(sfx_solver solver, double t, double* u, void* stream);
/* x = J(t, u_lin)^-1 rhs on the free vdofs with the essential rows/columns
 * eliminated; the essential entries of rhs are ignored and x is 0 there. */
int sfx_solver_solve_linear(sfx_solver solver, double t, const double* u_lin, const double* rhs, double* x,
                            void* stream);
/* x = J(t, u_lin)^-T rhs on the free vdofs (essential rows and columns
 * eliminated, x = 0 there): the adjoint solve, with the solver's Krylov
 * method and preconditioner applied to the transposed operator (the Jacobi
 * diagonal is the same; the learned network is used as trained).  Needs the
 * stored-tangent Jacobian mode. */
int sfx_solver_solve_adjoint(sfx_solver solver, double t, const double* u_lin, const double* rhs, double* x,
                             void* stream);
/* Load-step predictor: with d = u_target - u on the essential vdofs (0
 * elsewhere), solve J(t, u) x = -J(t, u) d on the free rows and set
 * u += d + x, so that u carries the new essential values and a first-order
 * response of the free vdofs to them (only the essential entries of
 * u_target are read).  Follow with sfx_solver_solve. */
int sfx_solver_warm_start(sfx_solver solver, double t, double* u, const double* u_target, void* stream);
int sfx_solver_get_stats(sfx_solver solver, sfx_solver_stats* out);
/* Network for SFX_PREC_LEARNED: the form's node grid (order * n + 1 nodes per
 * direction) and per-node features (device, [2][num_nodes] floats: log
 * modulus feature, Dirichlet mask), kept by reference. */
int sfx_solver_set_learned(sfx_solver solver, struct sfx_lnet_s* net, int nx, int ny, int nz, const float* features);

#ifdef __cplusplus
}
#endif

#endif /* SFX_SOLVER_H */
