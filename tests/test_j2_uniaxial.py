"""Known answer for J2 plasticity with linear hardening: serac's uniaxial
stress test (physics/materials/tests/J2_material.cpp:151-182), stated on a
unit cube.  Symmetry planes x = 0, y = 0, z = 0 and a prescribed stretch
u_x = eps on x = 1 give a homogeneous uniaxial stress state, which the H1
space reproduces exactly, so the x-reaction summed over the x = 1 face is
sigma_xx and the plastic strain at every quadrature point is the closed form:

    sigma_xx = E eps                          (eps < sigma_y / E)
             = E / (E + H) (sigma_y + H eps)  (otherwise)
    eps_p    = (E eps - sigma_y) / (E + H)

with E = 1, nu = 0.25, sigma_y = 0.01, H = E / 100, eps up to 2 sigma_y / E
in 4 steps, both checked to 1e-10 relative like the reference test.  The CPU
test runs the oracle (direct solves), the GPU test the device Newton solver."""
import numpy as np
import pytest

from oracle import oracle as O

E, NU, SY, H = 1.0, 0.25, 0.01, 0.01
STEPS = 4


def stress_exact(e):
    return E * e if e < SY / E else E / (E + H) * (SY + H * e)


def plastic_exact(e):
    return 0.0 if e < SY / E else (E * e - SY) / (E + H)


def _setup(n=2, p=1):
    m = O.StructuredHexMesh(n, n, n, O.box_vertices(n, n, n))
    N = m.num_nodes(p)
    x0, y0, z0 = (m.boundary_nodes(p, [s]) for s in (5, 2, 1))
    x1 = m.boundary_nodes(p, [3])
    ess = np.unique(np.concatenate([x0, N + y0, 2 * N + z0, x1]))
    return m, N, ess, x1


def _check(eps, reaction, qdata):
    assert abs(reaction - stress_exact(eps)) <= 1e-10 * abs(stress_exact(eps))
    pe = qdata[:, 0]  # plastic strain xx at every point
    if plastic_exact(eps) == 0.0:
        assert np.abs(pe).max() <= 1e-14
    else:
        assert np.abs(pe - plastic_exact(eps)).max() <= 1e-10 * plastic_exact(eps)


@pytest.mark.parametrize("p", [1, 2])
def test_uniaxial_oracle(p):
    m, N, ess, x1 = _setup(p=p)
    f = O.OracleFunctional(m, p, 3)
    f.add_domain_integral(O.MAT_J2, [E, NU, SY, H])
    u = np.zeros(f.ndofs)
    for k in range(1, STEPS + 1):
        eps = 2.0 * SY / E * k / STEPS
        target = np.zeros(f.ndofs)
        target[x1] = eps
        u = O.warm_start(f, u, target, ess)
        u, _, _ = O.newton(f, u, ess, rel_tol=1e-13, abs_tol=1e-15)
        r = f.residual(u, update_state=True)
        _check(eps, r[x1].sum(), f.state.reshape(-1, 10))


@pytest.mark.gpu
@pytest.mark.parametrize("p", [1, 2])
def test_uniaxial_device_solver(cuda, p):
    import torch

    import serac_gb300 as sg

    m, N, ess, x1 = _setup(p=p)
    mesh = sg.Mesh.structured_hex(2, 2, 2, m.vertices)
    f = sg.Functional(mesh, sg.H1(p, 3))
    f.AddDomainIntegral(sg.J2, [E, NU, SY, H])
    s = sg.NewtonSolver(f, sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, newton_rel_tol=1e-13,
                                                     newton_abs_tol=1e-16, krylov_rel_tol=1e-13,
                                                     krylov_abs_tol=1e-20, max_krylov_iterations=2000))
    s.set_essential(ess)
    u = torch.zeros(f.ndofs, dtype=torch.float64, device=cuda)
    for k in range(1, STEPS + 1):
        eps = 2.0 * SY / E * k / STEPS
        target = torch.zeros_like(u)
        target[torch.as_tensor(x1, device=cuda)] = eps
        s.warm_start(0.0, u, target)
        st = s.solve(0.0, u)
        assert st["converged"] == 1
        f.updateQdata(True)
        r = f.residual(0.0, u).cpu().numpy()
        f.updateQdata(False)
        _check(eps, r[x1].sum(), f.qdata().reshape(-1, 10))
