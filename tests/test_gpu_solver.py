"""Device Newton-Krylov solver against the oracle's Newton with direct solves.

Converged solutions agree to 1e-9 relative (the parity target for a converged
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


@pytest.mark.parametrize("precond", ["chebyshev", "mixed"])
def test_j2_load_steps_match_oracle(cuda, precond):
    """Small-strain J2 plasticity under compression in 4 load steps, each a
    warm-start predictor (SolidMechanics::warmStartDisplacement) followed by
    Newton; the plastic state is committed between steps.  The displacement
    and the quadrature state after every step match the oracle's direct-solve
    path to 1e-9."""
    import serac_gb300 as sg

    n, p, strain, steps = 3, 2, 0.02, 4
    V = O.box_vertices(n, n, n, 0.1, 1)
    m = O.StructuredHexMesh(n, n, n, V)
    orc = O.OracleFunctional(m, p, 3)
    orc.add_domain_integral(O.MAT_J2, [100.0, 0.3, 1.0, 1.0])
    mesh = sg.Mesh.structured_hex(n, n, n, V)
    f = sg.Functional(mesh, sg.H1(p, 3))
    f.AddDomainIntegral(sg.J2, [100.0, 0.3, 1.0, 1.0])
    N = f.num_nodes
    bottom, top = mesh.boundary_nodes(p, [1]), mesh.boundary_nodes(p, [6])
    ess = np.concatenate([bottom, N + bottom, 2 * N + bottom, 2 * N + top])
    kw = dict(newton_rel_tol=1e-11, newton_abs_tol=1e-13, krylov_rel_tol=1e-11, krylov_abs_tol=1e-18,
              max_krylov_iterations=3000)
    if precond == "mixed":
        kw["mixed_precision"] = 1
    s = sg.NewtonSolver(f, sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, **kw))
    s.set_essential(ess)
    u = torch.zeros(f.ndofs, dtype=torch.float64, device=cuda)
    uo = np.zeros(f.ndofs)
    for step in range(1, steps + 1):
        target = np.zeros(f.ndofs)
        target[2 * N + top] = -strain * step / steps
        s.warm_start(0.0, u, torch.tensor(target, device=cuda))
        st = s.solve(0.0, u)
        assert st["converged"] == 1 and st["newton_iterations"] <= 8
        uo = O.warm_start(orc, uo, target, ess)
        uo, _, _ = O.newton(orc, uo, ess, rel_tol=1e-12, abs_tol=1e-14)
        assert rel(u.cpu().numpy(), uo) <= 1e-9
        f.updateQdata(True)
        f.residual(0.0, u)
        f.updateQdata(False)
        orc.residual(uo, update_state=True)
        assert rel(f.qdata().reshape(-1, 10), orc.state.reshape(-1, 10)) <= 1e-8
    assert orc.state[..., 9].max() > 0.01  # the load drove the material well into plasticity
