"""Learned multilevel preconditioner (include/sfx_learned.h): network wrapper,
seeded heterogeneous material fields, training-data harvest from the solver
and training on the GPU with the library's own BF16 kernels.

    problems = [j2_problem(16, seed) for seed in range(1000, 1032)]
    R, T, F = harvest(problems)                     # (residual, correction) pairs + node features
    net = LearnedPreconditioner(seed=0)
    train(net, (33, 33, 33), R, T, F, epochs=40)
    S = SolidSetup(j2_problem(16, 2000))
    solver = NewtonSolver(S.f, SolverOptions.defaults(precond=LEARNED, mixed_precision=1))
    solver.set_essential(S.ess)
    solver.set_learned(net, S.grid, S.features)
    u, stats = solve_load_steps(S, solver)
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .functional import H1, Functional, Mesh, box_vertices
from .solver import JACOBI_CHEBYSHEV, NewtonSolver, SolverOptions  # noqa: F401 (re-exported for callers)


class LearnedPreconditioner:
    def __init__(self, seed: int = 0):
        h = ctypes.c_void_p()
        _lib.call("sfx_lnet_create", ctypes.c_uint64(seed), ctypes.byref(h))
        self._h = h
        n = ctypes.c_int64()
        _lib.call("sfx_lnet_num_params", h, ctypes.byref(n))
        self.num_params = n.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib._LIB is not None:
            _lib.load().sfx_lnet_destroy(self._h)
            self._h = None

    def params(self):
        p = np.zeros(self.num_params, dtype=np.float32)
        _lib.call("sfx_lnet_get_params", self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.size)
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _lib.call("sfx_lnet_set_params", self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.size)

    def save(self, path):
        np.save(path, self.params())

    def load(self, path):
        self.set_params(np.load(path))

    def apply(self, grid, r, features):
        nx, ny, nz = grid
        z = torch.empty_like(r)
        _lib.call("sfx_lnet_apply", self._h, nx, ny, nz, ctypes.c_void_p(r.data_ptr()),
                  ctypes.c_void_p(features.data_ptr()), ctypes.c_void_p(z.data_ptr()), None)
        return z

    def train_step(self, grid, R, T, F, batch, lr):
        nx, ny, nz = grid
        loss = ctypes.c_float()
        _lib.call("sfx_lnet_train_step", self._h, nx, ny, nz, batch, ctypes.c_void_p(R.data_ptr()),
                  ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(F.data_ptr()), ctypes.c_float(lr), ctypes.byref(loss),
                  None)
        return loss.value


# ------------------------------------------------------------- materials
def gaussian_random_field(n, ell, seed):
    """Unit-variance Gaussian random field on the n^3 element grid (element
    centroids on the unit cube) with Gaussian covariance exp(-|r|^2 / (2 ell^2))
    (correlation length ell), by spectral filtering of white noise: the
    covariance's spectral density is proportional to exp(-|k|^2 ell^2 / 2), so
    the noise is multiplied by its square root exp(-|k|^2 ell^2 / 4) (periodic
    FFT on a 2n grid, cropped to n).  tests/test_learned_host.py measures
    the correlation."""
    rng = np.random.default_rng(seed)
    m = 2 * n
    w = rng.standard_normal((m, m, m))
    k = 2 * np.pi * np.fft.fftfreq(m, d=1.0 / n)
    KZ, KY, KX = np.meshgrid(k, k, k, indexing="ij")
    S = np.exp(-(KX ** 2 + KY ** 2 + KZ ** 2) * ell ** 2 / 2.0)
    g = np.real(np.fft.ifftn(np.fft.fftn(w) * np.sqrt(S)))[:n, :n, :n]
    g = (g - g.mean()) / (g.std() + 1e-30)
    return g  # [z][y][x]


def node_features(n, order, elem_log_modulus, clamped_nodes, partial_nodes=()):
    """[2][num_nodes] float32: per-node mean of the incident elements' log
    modulus feature, and a constraint channel: 1 on fully clamped nodes (the
    network's output is zero there), 0.25 on partially constrained ones."""
    N1 = order * n + 1
    acc = np.zeros((N1, N1, N1))
    cnt = np.zeros((N1, N1, N1))
    f = elem_log_modulus.reshape(n, n, n)
    for dz in range(order + 1):
        for dy in range(order + 1):
            for dx in range(order + 1):
                acc[dz:dz + order * n:order, dy:dy + order * n:order, dx:dx + order * n:order] += f
                cnt[dz:dz + order * n:order, dy:dy + order * n:order, dx:dx + order * n:order] += 1
    feat = np.zeros(2 * N1 ** 3, dtype=np.float32)
    feat[:N1 ** 3] = (acc / cnt).ravel()
    feat[N1 ** 3 + np.asarray(partial_nodes, dtype=np.int64)] = 0.25
    feat[N1 ** 3 + np.asarray(clamped_nodes, dtype=np.int64)] = 1.0
    return feat


# --------------------------------------------------------------- problems
@dataclass
class SolidProblem:
    """Compression of the unit cube: z = 0 clamped, u_z = -strain on z = 1,
    per-element Young's modulus (J2) or shear modulus (Neo-Hookean)."""

    n: int
    material: int
    params: np.ndarray  # per-element parameters
    log_modulus: np.ndarray  # per-element feature
    strain: float
    steps: int
    perturb: float = 0.1
    seed: int = 1


def j2_problem(n, seed, sigma_log=None, ell=None, strain=0.02, steps=4):
    """Config-4 style problem: J2 small strain, E = 100 exp(sigma_log g),
    nu = 0.3, sigma_y = 1, H = 1; sigma_log in [0.5, 1.5], ell in [0.05, 0.3]
    drawn from the seed unless given."""
    from .functional import J2

    rng = np.random.default_rng(10_000 + seed)
    sigma_log = rng.uniform(0.5, 1.5) if sigma_log is None else sigma_log
    ell = rng.uniform(0.05, 0.3) if ell is None else ell
    g = gaussian_random_field(n, ell, seed).ravel()
    E = 100.0 * np.exp(sigma_log * g)
    params = np.stack([E, np.full_like(E, 0.3), np.ones_like(E), np.ones_like(E)], axis=1)
    return SolidProblem(n, J2, params, np.log(E / 100.0), strain, steps, seed=seed)


def neohookean_problem(n, seed, sigma_log=1.0, ell=0.1, strain=0.05, steps=10, bulk_ratio=20.0):
    """Config-3 style problem: shear modulus 0.25 exp(sigma_log g), K = 20 G."""
    from .functional import NEOHOOKEAN

    g = gaussian_random_field(n, ell, seed).ravel()
    G = 0.25 * np.exp(sigma_log * g)
    params = np.stack([bulk_ratio * G, G], axis=1)
    return SolidProblem(n, NEOHOOKEAN, params, np.log(G / 0.25), strain, steps, seed=seed)


class SolidSetup:
    """Form, Dirichlet data and features of a SolidProblem on the GPU."""

    def __init__(self, prob: SolidProblem, order=2):
        n = prob.n
        V = box_vertices(n, n, n, prob.perturb, prob.seed)
        self.mesh = Mesh.structured_hex(n, n, n, V)
        self.f = Functional(self.mesh, H1(order, 3))
        self.f.AddDomainIntegral(prob.material, prob.params, per_element=True)
        N = self.f.num_nodes
        bottom = self.mesh.boundary_nodes(order, [1])
        top = self.mesh.boundary_nodes(order, [6])
        self.ess = np.concatenate([bottom, N + bottom, 2 * N + bottom, 2 * N + top])
        self.top = top
        self.N = N
        self.grid = (order * n + 1,) * 3
        self.features = torch.tensor(node_features(n, order, prob.log_modulus, bottom, top), device="cuda")
        self.prob = prob

    def load(self, u, step):
        """Set the essential values of load step `step` in u."""
        u[2 * self.N + torch.as_tensor(self.top, device=u.device)] = -self.prob.strain * step / self.prob.steps

    def predictor(self, solver, u, step):
        """Warm-start u for load step `step` (SolidMechanics::warmStartDisplacement)."""
        target = u.clone()
        self.load(target, step)
        return solver.warm_start(0.0, u, target)

    def commit(self, u):
        """Commit the quadrature state of the converged step."""
        self.f.updateQdata(True)
        self.f.residual(0.0, u)
        self.f.updateQdata(False)


def solve_load_steps(setup, solver, u=None):
    """Quasi-static solve over the problem's load steps: predictor, Newton,
    state commit per step.  Returns u and the summed solver statistics."""
    u = torch.zeros(setup.f.ndofs, dtype=torch.float64, device="cuda") if u is None else u
    tot = {}
    for step in range(1, setup.prob.steps + 1):
        pre = setup.predictor(solver, u, step)
        st = solver.solve(0.0, u, raise_on_failure=False)
        for k, v in st.items():
            if k in ("converged",):
                tot[k] = min(tot.get(k, 1), v)
            elif isinstance(v, int):
                tot[k] = tot.get(k, 0) + v
        tot["predictor_krylov_iterations"] = tot.get("predictor_krylov_iterations", 0) + pre["krylov_iterations"]
        setup.commit(u)
    return u, tot


def smooth_fields(grid, count, rng, ell_range=(0.025, 0.25)):
    """count random 3-component displacement fields on the node grid: unit
    Gaussian random fields with a correlation length (Gaussian covariance
    exp(-r^2 / (2 ell^2)), unit cube) drawn from ell_range, byNODES float64
    [count, 3 * nodes]."""
    nx = grid[0]
    out = np.empty((count, 3 * nx ** 3))
    for i in range(count):
        ell = rng.uniform(*ell_range)
        for c in range(3):
            out[i, c * nx ** 3:(c + 1) * nx ** 3] = gaussian_random_field(nx, ell, int(rng.integers(2 ** 62))).ravel()
    return out


def probe_pairs(setup, u, count, rng):
    """Exact (residual, correction) pairs at the linearisation u: x a smooth
    random field with x = 0 on the essential vdofs, r = J(u) x with r = 0
    there.  Returns float32 CUDA tensors R, X [count, 3N]."""
    setup.f.linearize(0.0, u)
    ess = torch.as_tensor(setup.ess, device="cuda")
    X = torch.tensor(smooth_fields(setup.grid, count, rng), device="cuda")
    X[:, ess] = 0
    R = torch.empty_like(X)
    for i in range(count):
        setup.f.gradient.mult(X[i].contiguous(), out=R[i])
    R[:, ess] = 0
    return R.float(), X.float()


def harvest(problems, order=2, options=None, probes_per_step=8, newton_pairs=True, max_newton_pairs=64, seed=0,
            log=None):
    """Training pairs from the solver on each problem's load steps (warm
    start, Newton with the FP32-inner mixed-precision solve, state commit):
    every Newton step's (residual, correction) pair, and probes_per_step
    probe pairs at each converged step.  Returns float32 CUDA tensors
    R, T [pairs, 3N] and F [pairs, 2N].  log(problems_done, pairs) is called
    after every problem when given."""
    from .solver import SolverOptions as _SO

    opts = options or _SO.defaults(precond=JACOBI_CHEBYSHEV, mixed_precision=1, krylov_rel_tol=1e-6,
                                   max_krylov_iterations=1000)
    rng = np.random.default_rng(seed)
    Rs, Ts, Fs = [], [], []
    for done, prob in enumerate(problems, 1):
        S = SolidSetup(prob, order)
        solver = NewtonSolver(S.f, opts)
        solver.set_essential(S.ess)
        ess = torch.as_tensor(S.ess, device="cuda")
        u = torch.zeros(S.f.ndofs, dtype=torch.float64, device="cuda")
        count = 0
        for step in range(1, prob.steps + 1):
            S.predictor(solver, u, step)
            r = S.f.residual(0.0, u)
            r[ess] = 0
            r0 = float(torch.linalg.norm(r))
            for _ in range(10):
                rn = float(torch.linalg.norm(r))
                if rn <= 1e-8 * r0 or rn <= 1e-14:
                    break
                du = solver.solve_linear(0.0, u, r)
                if newton_pairs and count < max_newton_pairs:
                    Rs.append(r.float().clone())
                    Ts.append(du.float().clone())
                    Fs.append(S.features)
                    count += 1
                u -= du
                r = S.f.residual(0.0, u)
                r[ess] = 0
            if probes_per_step:
                R, X = probe_pairs(S, u, probes_per_step, rng)
                Rs.extend(R)
                Ts.extend(X)
                Fs.extend([S.features] * probes_per_step)
            S.commit(u)
        if log is not None:
            log(done, len(Rs))
    return torch.stack(Rs), torch.stack(Ts), torch.stack(Fs)


def train(net, grid, R, T, F, epochs=20, batch=8, lr=1e-3, lr_min=None, warmup=0.05, seed=0, log=None):
    """Adam over shuffled mini-batches of the pairs; the learning rate rises
    linearly over the first `warmup` fraction of the steps, then decays from lr
    to lr_min (default lr / 20) on a cosine.  Returns the mean loss of every
    epoch."""
    rng = np.random.default_rng(seed)
    n = R.shape[0]
    lr_min = lr / 20 if lr_min is None else lr_min
    steps = max(1, epochs * (n // batch))
    n_warm = max(1, int(warmup * steps))
    hist, k = [], 0
    for ep in range(epochs):
        order = rng.permutation(n)
        tot = 0.0
        for i in range(0, n - batch + 1, batch):
            idx = torch.as_tensor(order[i:i + batch], device=R.device)
            Rb, Tb, Fb = R[idx].contiguous(), T[idx].contiguous(), F[idx].contiguous()
            if k < n_warm:
                lr_k = lr * (k + 1) / n_warm
            else:
                lr_k = lr_min + 0.5 * (lr - lr_min) * (1.0 + np.cos(np.pi * (k - n_warm) / max(1, steps - n_warm)))
            tot += net.train_step(grid, Rb, Tb, Fb, batch, lr_k)
            k += 1
        hist.append(tot / max(1, n // batch))
        if log:
            log(ep, hist[-1])
    return hist
