"""Failure detection without faulting the GPU: every failure is made on the
host (corrupted inputs, an impossible operator, an iteration cap) or by a
device wait that is bounded by construction, and each must come back as a
status code with the context still usable."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _solid(n=3, params=None, per_element=False):
    import serac_gb300 as sg

    V = O.box_vertices(n, n, n, 0.1, 1)
    mesh = sg.Mesh.structured_hex(n, n, n, V)
    f = sg.Functional(mesh, sg.H1(2, 3))
    f.AddDomainIntegral(sg.NEOHOOKEAN, [5.0, 0.25] if params is None else params, per_element=per_element)
    N = f.num_nodes
    bottom, top = mesh.boundary_nodes(2, [1]), mesh.boundary_nodes(2, [6])
    ess = np.concatenate([bottom, N + bottom, 2 * N + bottom, 2 * N + top])
    u = torch.zeros(f.ndofs, dtype=torch.float64, device="cuda")
    u[2 * N + torch.as_tensor(top, device="cuda")] = -0.01
    return f, ess, u


def test_bounded_device_wait_expires_with_a_status(cuda):
    """A block waits on an mbarrier that nothing completes (the wait helper of
    the bulk-copy kernels, bounded to 2000 polls): SFX_ERR_TIMEOUT, and the
    next computation on the same context still matches the oracle."""
    from serac_gb300 import _lib

    rc = _lib.load().sfx_selftest_bounded_wait(2000)
    assert rc == -4  # SFX_ERR_TIMEOUT
    f, _, u = _solid()
    r = f.residual(0.0, u)
    assert bool(torch.isfinite(r).all())


def test_nonfinite_material_parameter_gives_status(cuda):
    import serac_gb300 as sg
    from serac_gb300._lib import SfxError

    params = np.tile([5.0, 0.25], (27, 1))
    params[13, 1] = np.nan  # one corrupted element
    f, ess, u = _solid(params=params, per_element=True)
    s = sg.NewtonSolver(f)
    s.set_essential(ess)
    with pytest.raises(SfxError) as e:
        s.solve(0.0, u)
    assert e.value.code == -3  # SFX_ERR_NONFINITE


def test_nonfinite_state_gives_status_and_solver_recovers(cuda):
    import serac_gb300 as sg
    from serac_gb300._lib import SfxError

    f, ess, u = _solid()
    s = sg.NewtonSolver(f, sg.SolverOptions.defaults(newton_abs_tol=1e-16))
    s.set_essential(ess)
    bad = u.clone()
    bad[5] = float("inf")
    with pytest.raises(SfxError) as e:
        s.solve(0.0, bad)
    assert e.value.code == -3
    st = s.solve(0.0, u)  # the same solver, clean input
    assert st["converged"] == 1


def test_zero_right_hand_side(cuda):
    import serac_gb300 as sg

    f, ess, u = _solid()
    s = sg.NewtonSolver(f)
    s.set_essential(ess)
    x = s.solve_linear(0.0, u, torch.zeros_like(u))
    assert float(x.abs().max()) == 0.0
    assert s.stats()["krylov_iterations"] == 0


def test_cg_breakdown_gives_status(cuda):
    """CG on a negative-definite operator (conductivity -1) breaks down at the
    first step: a status, not a trap."""
    import serac_gb300 as sg
    from serac_gb300._lib import SfxError

    n = 3
    mesh = sg.Mesh.structured_hex(n, n, n, O.box_vertices(n, n, n))
    f = sg.Functional(mesh, sg.H1(2, 1))
    f.AddDomainIntegral(sg.HEAT, [-1.0, 1.0])
    s = sg.NewtonSolver(f, sg.SolverOptions.defaults(krylov=sg.CG, precond=sg.JACOBI))
    s.set_essential(mesh.boundary_nodes(2, [5]))
    u = torch.zeros(f.ndofs, dtype=torch.float64, device="cuda")
    with pytest.raises(SfxError) as e:
        s.solve(0.0, u)
    assert e.value.code == -3 and "CG breakdown" in str(e.value)


def test_newton_iteration_cap_gives_status(cuda):
    import serac_gb300 as sg
    from serac_gb300._lib import SfxError

    f, ess, u = _solid()
    s = sg.NewtonSolver(f, sg.SolverOptions.defaults(max_newton_iterations=1, newton_rel_tol=1e-14,
                                                     newton_abs_tol=1e-30))
    s.set_essential(ess)
    with pytest.raises(SfxError) as e:
        s.solve(0.0, u.clone())
    assert e.value.code == -7  # SFX_ERR_NOT_CONVERGED
    st = s.solve(0.0, u.clone(), raise_on_failure=False)
    assert st["converged"] == 0 and st["newton_iterations"] == 1
