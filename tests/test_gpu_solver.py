"""Device Newton-Krylov solver against the oracle's Newton with direct solves.

Converged solutions agree to 1e-9 relative (spec parity target for the
Newton solution); every Krylov / preconditioner combination must reach the
same answer, including the FP32-inner mixed-precision mode.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import rel

pytestmark = pytest.mark.gpu


def _heat(n=6, p=2):
    import serac_gb300 as sg

    V = O.box_vertices(n, n, n, 0.1, 3)
    m = O.StructuredHexMesh(n, n, n, V)
    orc = O.OracleFunctional(m, p, 1)
    orc.add_domain_integral(O.MAT_HEAT, [1.0, 1.0])
    mesh = sg.Mesh.structured_hex(n, n, n, V)
    f = sg.Functional(mesh, sg.H1(p, 1))
    f.AddDomainIntegral(sg.HEAT, [1.0, 1.0])
    ess = mesh.boundary_nodes(p, [5])  # x = 0
    return orc, f, mesh, ess


def _solid(n=4, p=2, uz=-0.02):
    import serac_gb300 as sg

    V = O.box_vertices(n, n, n, 0.1, 1)
    m = O.StructuredHexMesh(n, n, n, V)
    orc = O.OracleFunctional(m, p, 3)
    orc.add_domain_integral(O.MAT_NEOHOOKEAN, [5.0, 0.25])
    mesh = sg.Mesh.structured_hex(n, n, n, V)
    f = sg.Functional(mesh, sg.H1(p, 3))
    f.AddDomainIntegral(sg.NEOHOOKEAN, [5.0, 0.25])
    N = f.num_nodes
    bottom = mesh.boundary_nodes(p, [1])
    top = mesh.boundary_nodes(p, [6])
    ess = np.concatenate([bottom, N + bottom, 2 * N + bottom, 2 * N + top])
    u0 = np.zeros(f.ndofs)
    u0[2 * N + top] = uz
    return orc, f, ess, u0


def test_heat_cg_matches_direct_solve(cuda):
    import serac_gb300 as sg

    orc, f, mesh, ess = _heat()
    opts = sg.SolverOptions.defaults(krylov=sg.CG, precond=sg.JACOBI, krylov_rel_tol=1e-13, newton_rel_tol=1e-11)
    s = sg.NewtonSolver(f, opts)
    s.set_essential(ess)
    u = torch.zeros(f.ndofs, dtype=torch.float64, device=cuda)
    st = s.solve(0.0, u)
    assert st["converged"] == 1 and st["newton_iterations"] == 1
    ref, _, _ = O.newton(orc, np.zeros(f.ndofs), ess)
    assert rel(u.cpu().numpy(), ref) <= 1e-9


@pytest.mark.parametrize("precond", ["jacobi", "chebyshev", "mixed"])
def test_neohookean_newton_matches_oracle(cuda, precond):
    import serac_gb300 as sg

    orc, f, ess, u0 = _solid()
    kw = dict(newton_rel_tol=1e-12, newton_abs_tol=1e-16, krylov_rel_tol=1e-10, krylov_abs_tol=1e-16,
              max_krylov_iterations=2000)
    if precond == "jacobi":
        kw.update(precond=sg.JACOBI)
    elif precond == "mixed":
        kw.update(precond=sg.JACOBI_CHEBYSHEV, mixed_precision=1)
    opts = sg.SolverOptions.defaults(**kw)
    s = sg.NewtonSolver(f, opts)
    s.set_essential(ess)
    u = torch.tensor(u0, device=cuda)
    st = s.solve(0.0, u)
    assert st["converged"] == 1
    ref, it, _ = O.newton(orc, u0, ess, rel_tol=1e-13, abs_tol=1e-16)
    assert rel(u.cpu().numpy(), ref) <= 1e-9
    # the solution satisfies the equations to the requested tolerance
    r = orc.residual(u.cpu().numpy())
    r[ess] = 0
    r0 = orc.residual(u0)
    r0[ess] = 0
    assert np.linalg.norm(r) <= 1e-11 * np.linalg.norm(r0)
    if precond == "mixed":
        assert st["inner_iterations"] > 0


def test_solve_linear_matches_direct(cuda):
    import serac_gb300 as sg

    orc, f, ess, u0 = _solid(n=3)
    rng = np.random.default_rng(4)
    ul = u0 + 0.002 * rng.standard_normal(f.ndofs)
    ul[ess] = u0[ess]
    b = rng.standard_normal(f.ndofs)
    b[ess] = 0
    s = sg.NewtonSolver(f, sg.SolverOptions.defaults(krylov_rel_tol=1e-12, max_krylov_iterations=3000))
    s.set_essential(ess)
    x = s.solve_linear(0.0, torch.tensor(ul, device=cuda), torch.tensor(b, device=cuda)).cpu().numpy()
    import scipy.sparse.linalg as spla

    A = O.eliminate_dirichlet(orc.assemble(ul), ess)
    ref = spla.spsolve(A.tocsc(), b)
    assert rel(x, ref) <= 1e-9


def test_solver_is_bitwise_reproducible(cuda):
    import serac_gb300 as sg

    _, f, ess, u0 = _solid(n=3)
    outs = []
    for _ in range(2):
        s = sg.NewtonSolver(f, sg.SolverOptions.defaults(mixed_precision=1))
        s.set_essential(ess)
        u = torch.tensor(u0, device=cuda)
        s.solve(0.0, u)
        outs.append(u.clone())
    assert torch.equal(outs[0], outs[1])
