"""Adjoint shape sensitivities on the GPU: (dR/dp)^T lam (sfx_shape_vjp)
against the forward shape derivative (adjoint identity, 1e-12) and against
central differences of the oracle's residual; dQ/dp of quantities of
interest against central differences of the oracle and the exact rates of a
dilation; and the total derivative dQ/dp - lam^T dR/dp of a solved heat
problem against finite differences of Q(u*(p), p)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import PARAMS, mesh, rel

pytestmark = pytest.mark.gpu

VCASES = [
    # (material, p, boundary integral or None)
    (O.MAT_HEAT, 1, None),
    (O.MAT_HEAT, 2, (O.BMAT_HEAT_FLUX, (1, 3, 6), [0.3, 0.7, 1.1])),
    (O.MAT_NONLINEAR_HEAT, 1, (O.BMAT_HEAT_FLUX, (2, 5), [0.1, -0.2, 0.5])),
    (O.MAT_NEOHOOKEAN, 2, (O.BMAT_PRESSURE, (3, 6), [0.7])),
    (O.MAT_NEOHOOKEAN, 1, (O.BMAT_TRACTION, (4,), [0.1, 0.2, 0.3, 0.5, -0.4, 0.2])),
    (O.MAT_J2, 2, None),
    (O.MAT_THERMAL_TEST, 2, None),
]


def _pair(mat, p, bnd, dims=(3, 2, 2), seed=5):
    import serac_gb300 as sg

    m = mesh(*dims, perturb=0.1, seed=seed)
    c = O.COMPONENTS[mat]
    orc = O.OracleFunctional(m, p, c)
    f = sg.Functional(sg.Mesh.structured_hex(*dims, m.vertices), sg.H1(p, c))
    orc.add_domain_integral(mat, PARAMS[mat])
    f.AddDomainIntegral(mat, PARAMS[mat])
    if bnd is not None:
        orc.add_boundary_integral(*bnd)
        f.AddBoundaryIntegral(*bnd)
    return m, orc, f


@pytest.mark.parametrize("case", range(len(VCASES)))
def test_shape_vjp_adjoint_identity(cuda, case):
    """<lam, (dR/dp) dp> = <(dR/dp)^T lam, dp> on a shape-displaced configuration."""
    import serac_gb300 as sg

    mat, p, bnd = VCASES[case]
    m, orc, f = _pair(mat, p, bnd)
    rng = np.random.default_rng(60 + case)
    nn = m.num_nodes(p)
    shape = torch.tensor(rng.standard_normal(3 * nn) * 0.01, device=cuda)
    u = torch.tensor(rng.standard_normal(f.ndofs) * (0.02 if O.COMPONENTS[mat] == 3 else 0.3), device=cuda)
    lam = torch.tensor(rng.standard_normal(f.ndofs), device=cuda)
    dp = torch.tensor(rng.standard_normal(3 * nn), device=cuda)
    f.set_shape_displacement(shape)
    dRdp = sg.ShapeGradient(f, 0.0, u)
    fwd = dRdp(dp)
    vjp = dRdp.MultTranspose(lam)
    lhs = float(torch.dot(lam, fwd))
    rhs = float(torch.dot(vjp, dp))
    scale = float(torch.linalg.norm(lam) * torch.linalg.norm(fwd))
    assert abs(lhs - rhs) <= 1e-12 * scale


@pytest.mark.parametrize("case", [0, 1, 3])
def test_shape_vjp_finite_differences(cuda, case):
    import serac_gb300 as sg

    mat, p, bnd = VCASES[case]
    m, orc, f = _pair(mat, p, bnd, dims=(2, 2, 1), seed=7)
    rng = np.random.default_rng(70 + case)
    nn = m.num_nodes(p)
    shape = rng.standard_normal(3 * nn) * 0.01
    u = rng.standard_normal(f.ndofs) * (0.02 if O.COMPONENTS[mat] == 3 else 0.3)
    lam = rng.standard_normal(f.ndofs)
    f.set_shape_displacement(torch.tensor(shape, device=cuda))
    g = sg.ShapeGradient(f, 0.0, torch.tensor(u, device=cuda))
    got = g.MultTranspose(torch.tensor(lam, device=cuda)).cpu().numpy()
    ref = orc.shape_vjp_fd(u, lam, base_shape=shape, h=1e-6)
    assert rel(got, ref) <= 1e-6


QCASES = [
    (1, 1, [(O.QOI_MEASURE, None), (O.QOI_POLY_TEST, None)], [(O.QOI_POLY_TEST, [1, 3, 6], None)]),
    (2, 1, [(O.QOI_POSITION, [1.0, -2.0, 0.5])], [(O.QOI_MEASURE, [2, 4, 5], None)]),
    (2, 3, [(O.QOI_NEOHOOKEAN_ENERGY, [5.0, 0.25])], [(O.QOI_NORMAL_FIELD, [6], None)]),
    (1, 3, [(O.QOI_FIELD, [1.0, 2.0, -1.0])], [(O.QOI_POLY_TEST, [2, 5], None)]),
]


@pytest.mark.parametrize("case", range(len(QCASES)))
def test_qoi_shape_gradient_finite_differences(cuda, case):
    import serac_gb300 as sg

    p, c, domain, faces = QCASES[case]
    dims = (2, 2, 1)
    m = mesh(*dims, perturb=0.1, seed=9)
    rng = np.random.default_rng(80 + case)
    nn = m.num_nodes(p)
    shape = rng.standard_normal(3 * nn) * 0.01
    amp = 0.01 if any(k == O.QOI_NEOHOOKEAN_ENERGY for k, _ in domain) else 0.1
    u = rng.standard_normal(nn * c) * amp
    orc = O.OracleQoI(m, p, c, shape=shape)
    q = sg.QoI(sg.Mesh.structured_hex(*dims, m.vertices), sg.H1(p, c))
    for kind, params in domain:
        orc.add_domain_integral(kind, params)
        q.AddDomainIntegral(kind, params)
    for kind, sides, params in faces:
        orc.add_boundary_integral(kind, sides, params)
        q.AddBoundaryIntegral(kind, sides, params)
    q.set_shape_displacement(torch.tensor(shape, device=cuda))
    got = q.shape_gradient(0.0, torch.tensor(u, device=cuda)).cpu().numpy()
    ref = orc.shape_gradient_fd(u, base_shape=shape, h=1e-6)
    assert rel(got, ref) <= 1e-6


def test_qoi_shape_gradient_dilation(cuda):
    """Exact rates: a dilation p = eps X changes the volume at 3 V, the
    surface area at 2 A; translations change neither."""
    import serac_gb300 as sg

    m = mesh(4, 3, 2, perturb=0.2, seed=3)
    M = sg.Mesh.structured_hex(4, 3, 2, m.vertices)
    for p in (1, 2):
        X = m.node_coordinates(p)
        dil = torch.tensor(np.concatenate([X[:, 0], X[:, 1], X[:, 2]]), device=cuda)
        trans = torch.tensor(np.repeat([0.3, -0.1, 0.2], len(X)), device=cuda)
        u = torch.zeros(len(X), dtype=torch.float64, device=cuda)
        vol = sg.QoI(M, sg.H1(p, 1))
        vol.AddDomainIntegral(sg.QOI_MEASURE)
        gv = vol.shape_gradient(0.0, u)
        assert abs(float(torch.dot(gv, dil)) - 3.0) <= 1e-12
        assert abs(float(torch.dot(gv, trans))) <= 1e-12
        area = sg.QoI(M, sg.H1(p, 1))
        area.AddBoundaryIntegral(sg.QOI_MEASURE, [1, 2, 3, 4, 5, 6])
        ga = area.shape_gradient(0.0, u)
        assert abs(float(torch.dot(ga, dil)) - 12.0) <= 1e-11
        assert abs(float(torch.dot(ga, trans))) <= 1e-12


def test_total_shape_sensitivity_by_adjoint(cuda):
    """Heat conduction with u = 0 on x = 0 and a source: the total derivative
    of Q = int u over the solved state, dQ/dp - lam^T dR/dp with
    J^T lam = dQ/du, against central differences of Q(u*(p), p)."""
    import serac_gb300 as sg

    dims = (4, 3, 3)
    p = 2
    m = mesh(*dims, perturb=0.1, seed=11)
    M = sg.Mesh.structured_hex(*dims, m.vertices)
    f = sg.Functional(M, sg.H1(p, 1))
    f.AddDomainIntegral(sg.HEAT, [1.3, 0.7])
    f.AddBoundaryIntegral(sg.HEAT_FLUX, [3], [0.2, 0.1, 0.5])
    q = sg.QoI(M, sg.H1(p, 1))
    q.AddDomainIntegral(sg.QOI_FIELD, [1.0])
    q.AddBoundaryIntegral(sg.QOI_POLY_TEST, [6])
    ess = m.boundary_nodes(p, [5])
    opts = sg.SolverOptions.defaults(krylov=sg.GMRES, precond=sg.JACOBI, krylov_rel_tol=1e-13, krylov_abs_tol=0.0,
                                     newton_rel_tol=1e-12, newton_abs_tol=0.0)
    solver = sg.NewtonSolver(f, opts)
    solver.set_essential(ess)
    nn = m.num_nodes(p)
    X = m.node_coordinates(p)
    # smooth shape direction that keeps the Dirichlet side in place
    dp = np.concatenate([0.05 * X[:, 0] * np.sin(np.pi * X[:, 1]), 0.03 * X[:, 0] * X[:, 2], 0.02 * X[:, 0] ** 2])
    dp_t = torch.tensor(dp, device=cuda)

    def solve_at(shape):
        f.set_shape_displacement(shape)
        q.set_shape_displacement(shape)
        u = torch.zeros(nn, dtype=torch.float64, device=cuda)
        solver.solve(0.0, u)
        return u

    zero = torch.zeros(3 * nn, dtype=torch.float64, device=cuda)
    u0 = solve_at(zero)
    dQdu = q.gradient(0.0, u0)
    lam = solver.solve_adjoint(0.0, u0, dQdu)
    dQdp = q.shape_gradient(0.0, u0)
    vjp = sg.ShapeGradient(f, 0.0, u0).MultTranspose(lam)
    total = dQdp - vjp
    pred = float(torch.dot(total, dp_t))
    h = 1e-4
    qp = q(0.0, solve_at(h * dp_t))
    qm = q(0.0, solve_at(-h * dp_t))
    fd = (qp - qm) / (2 * h)
    assert abs(pred - fd) <= 1e-6 * abs(fd)
    assert abs(float(torch.dot(dQdp, dp_t))) > 1e-3 * abs(fd)  # both terms matter
