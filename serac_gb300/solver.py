"""Device-resident Newton-Krylov solver (include/sfx_solver.h) for a Functional.

    solver = NewtonSolver(f, SolverOptions(krylov=GMRES, precond=JACOBI_CHEBYSHEV))
    solver.set_essential(dofs)          # Dirichlet vdofs; values taken from u
    stats = solver.solve(t, u)          # u: float64 CUDA tensor, updated in place

Mirrors serac's EquationSolver / NewtonSolver (equation_solver.cpp:79-200,
820-950) with the options of solver_config.hpp:342-400, plus the
Jacobi-Chebyshev, flexible-GMRES and FP32-inner mixed-precision modes.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .functional import Functional, _dptr, _require, _stream

GMRES, CG, FGMRES = 0, 1, 2
NONE, JACOBI, JACOBI_CHEBYSHEV, LEARNED = 0, 1, 2, 3
ERR_NOT_CONVERGED = -7


class SolverOptions(ctypes.Structure):
    _fields_ = [
        ("max_newton_iterations", ctypes.c_int),
        ("newton_rel_tol", ctypes.c_double),
        ("newton_abs_tol", ctypes.c_double),
        ("krylov", ctypes.c_int),
        ("restart", ctypes.c_int),
        ("max_krylov_iterations", ctypes.c_int),
        ("krylov_rel_tol", ctypes.c_double),
        ("krylov_abs_tol", ctypes.c_double),
        ("precond", ctypes.c_int),
        ("chebyshev_degree", ctypes.c_int),
        ("chebyshev_ratio", ctypes.c_double),
        ("eigen_iterations", ctypes.c_int),
        ("mixed_precision", ctypes.c_int),
        ("inner_iterations", ctypes.c_int),
        ("inner_rel_tol", ctypes.c_double),
        ("print_level", ctypes.c_int),
        ("learned_cycle", ctypes.c_int),
        ("inner_chebyshev_degree", ctypes.c_int),
        ("learned_max_rejections", ctypes.c_int),
    ]

    @classmethod
    def defaults(cls, **kw):
        o = cls()
        _lib.call("sfx_solver_default_options", ctypes.addressof(o))
        for k, v in kw.items():
            if not hasattr(o, k):
                raise AttributeError(k)
            setattr(o, k, v)
        return o


class SolverStats(ctypes.Structure):
    _fields_ = [
        ("newton_iterations", ctypes.c_int),
        ("krylov_iterations", ctypes.c_int),
        ("inner_iterations", ctypes.c_int),
        ("converged", ctypes.c_int),
        ("initial_residual", ctypes.c_double),
        ("final_residual", ctypes.c_double),
        ("last_krylov_rel", ctypes.c_double),
        ("learned_applications", ctypes.c_int),
        ("learned_fallbacks", ctypes.c_int),
        ("lmax_estimate", ctypes.c_double),
        ("learned_skipped", ctypes.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class NewtonSolver:
    def __init__(self, form: Functional, options: SolverOptions | None = None):
        _lib.load()
        self.form = form
        self.options = options if options is not None else SolverOptions.defaults()
        h = ctypes.c_void_p()
        _lib.call("sfx_solver_create", form._h, ctypes.addressof(self.options), ctypes.byref(h))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib._LIB is not None:
            _lib.load().sfx_solver_destroy(self._h)
            self._h = None

    def set_essential(self, dofs):
        d = np.ascontiguousarray(np.asarray(dofs, dtype=np.int64).ravel())
        self._ess = d
        _lib.call("sfx_solver_set_essential", self._h, d.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), d.size)

    def set_learned(self, net, grid, features):
        """Use a LearnedPreconditioner (precond=LEARNED): grid = node grid
        (nx, ny, nz), features = float32 CUDA tensor [2 * num_nodes]."""
        if not (isinstance(features, torch.Tensor) and features.is_cuda and features.dtype == torch.float32):
            raise TypeError("features must be a float32 CUDA tensor")
        self._features = features
        self._net = net
        _lib.call("sfx_solver_set_learned", self._h, net._h, int(grid[0]), int(grid[1]), int(grid[2]),
                  _dptr(features))

    def stats(self):
        st = SolverStats()
        _lib.call("sfx_solver_get_stats", self._h, ctypes.addressof(st))
        return st.as_dict()

    def solve(self, t, u, stream=None, raise_on_failure=True):
        _require(u, torch.float64, self.form.ndofs, "u")
        rc = _lib.load().sfx_solver_solve(self._h, float(t), _dptr(u), _stream(stream))
        if rc != 0 and (raise_on_failure or rc != ERR_NOT_CONVERGED):
            _lib.check(rc)
        return self.stats()

    def warm_start(self, t, u, u_target, stream=None):
        """Load-step predictor (SolidMechanics::warmStartDisplacement): moves
        the essential vdofs of u to u_target's values and the free vdofs by
        the linearised response to that change."""
        _require(u, torch.float64, self.form.ndofs, "u")
        _require(u_target, torch.float64, self.form.ndofs, "u_target")
        _lib.call("sfx_solver_warm_start", self._h, float(t), _dptr(u), _dptr(u_target), _stream(stream))
        return self.stats()

    def solve_linear(self, t, u_lin, rhs, out=None, stream=None):
        _require(u_lin, torch.float64, self.form.ndofs, "u_lin")
        _require(rhs, torch.float64, self.form.ndofs, "rhs")
        out = torch.empty_like(rhs) if out is None else out
        _lib.call("sfx_solver_solve_linear", self._h, float(t), _dptr(u_lin), _dptr(rhs), _dptr(out), _stream(stream))
        return out

    def solve_adjoint(self, t, u_lin, rhs, out=None, stream=None):
        """lambda = J(t, u_lin)^-T rhs on the free vdofs (0 on the essential
        set): the adjoint solve of SolidMechanics::reverseAdjointTimestep
        (solid_mechanics.hpp:1343-1501), matrix-free with the transposed action."""
        _require(u_lin, torch.float64, self.form.ndofs, "u_lin")
        _require(rhs, torch.float64, self.form.ndofs, "rhs")
        out = torch.empty_like(rhs) if out is None else out
        _lib.call("sfx_solver_solve_adjoint", self._h, float(t), _dptr(u_lin), _dptr(rhs), _dptr(out),
                  _stream(stream))
        return out
