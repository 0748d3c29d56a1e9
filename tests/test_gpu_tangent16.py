"""The FP16 copy of the stored tangent for the FP32 action (the inner Krylov
operator of the mixed-precision solver): the action against the FP64
oracle to the precision of FP16 entries, transposed too, and a mixed-precision
Newton solve that reaches the plain FP64 answer (the outer FP64 FGMRES
corrects the inner operator's rounding)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import PARAMS, mesh, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mat", [O.MAT_NEOHOOKEAN, O.MAT_J2, O.MAT_THERMAL_TEST, O.MAT_HEAT])
def test_fp16_tangent_action(cuda, mat):
    import serac_gb300 as sg

    m = mesh(3, 2, 2, perturb=0.1, seed=5)
    c = O.COMPONENTS[mat]
    orc = O.OracleFunctional(m, 2, c)
    orc.add_domain_integral(mat, PARAMS[mat])
    f = sg.Functional(sg.Mesh.structured_hex(3, 2, 2, m.vertices), sg.H1(2, c))
    f.AddDomainIntegral(mat, PARAMS[mat])
    f.set_tangent_storage(f.TANGENT_F16)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(orc.ndofs) * (0.02 if c == 3 else 0.3)
    du = rng.standard_normal(orc.ndofs)
    _, g = f(0.0, sg.differentiate_wrt(torch.tensor(u, device=cuda)))
    dut = torch.tensor(du, device=cuda)
    ref = orc.jvp(u, du)
    assert rel(g(dut).cpu().numpy(), ref) <= 1e-12  # FP64 untouched
    err = rel(g(dut.float()).double().cpu().numpy(), ref)
    assert 1e-7 < err <= 3e-3  # FP16 entries, FP32 accumulation
    assert rel(g.MultTranspose(dut.float()).double().cpu().numpy(), orc.jvp_transpose(u, du)) <= 3e-3


def test_fp16_tangent_order1_unsupported(cuda):
    import serac_gb300 as sg
    from serac_gb300._lib import SfxError

    m = mesh(2, 2, 2)
    f = sg.Functional(sg.Mesh.structured_hex(2, 2, 2, m.vertices), sg.H1(1, 1))
    with pytest.raises(SfxError):
        f.set_tangent_storage(f.TANGENT_F16)


def test_fp16_tangent_mixed_newton(cuda):
    """J2 load step on 8^3 Q2: mixed precision with the FP16 inner tangent
    reaches the plain FP64 solution."""
    import serac_gb300 as sg
    from serac_gb300 import learned as LP

    prob = LP.j2_problem(8, 2000)
    base = dict(newton_rel_tol=1e-10, newton_abs_tol=0.0, krylov_rel_tol=1e-10, krylov_abs_tol=0.0,
                max_krylov_iterations=5000)
    sols = []
    for f16, opts in ((False, sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, **base)),
                      (True, sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, mixed_precision=1, **base))):
        S = LP.SolidSetup(prob)
        if f16:
            S.f.set_tangent_storage(S.f.TANGENT_F16)
        solver = sg.NewtonSolver(S.f, opts)
        solver.set_essential(S.ess)
        u = torch.zeros(S.f.ndofs, dtype=torch.float64, device=cuda)
        S.predictor(solver, u, 1)
        st = solver.solve(0.0, u)
        assert st["converged"] == 1
        sols.append(u.cpu().numpy())
    assert rel(sols[1], sols[0]) <= 1e-8
