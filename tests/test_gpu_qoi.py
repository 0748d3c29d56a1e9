"""Quantities of interest (Functional<double(H1<p,c>)>) and transposed
Jacobian actions on the GPU against the oracle: values, directional
derivatives and gradients of domain and face integrands (with and without a
shape displacement); J^T v for symmetric and non-symmetric operators (FP64 to
1e-12, FP32 to 1e-5); the adjoint identity at the 32^3 Neo-Hookean size; and
the adjoint solve."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import PARAMS, mesh, rel

pytestmark = pytest.mark.gpu

ALL_SIDES = [1, 2, 3, 4, 5, 6]


def _qoi_pair(p, c, domain, faces, dims=(3, 2, 2), shape_amp=0.0, seed=5):
    import serac_gb300 as sg

    m = mesh(*dims, perturb=0.1, seed=seed)
    shape = None
    if shape_amp:
        shape = np.random.default_rng(seed + 1).standard_normal(3 * m.num_nodes(p)) * shape_amp
    orc = O.OracleQoI(m, p, c, shape=shape)
    q = sg.QoI(sg.Mesh.structured_hex(*dims, m.vertices), sg.H1(p, c))
    for kind, params in domain:
        orc.add_domain_integral(kind, params)
        q.AddDomainIntegral(kind, params)
    for kind, sides, params in faces:
        orc.add_boundary_integral(kind, sides, params)
        q.AddBoundaryIntegral(kind, sides, params)
    if shape is not None:
        q.set_shape_displacement(torch.tensor(shape, device="cuda"))
    return orc, q


CASES = [
    # (p, c, domain integrals, face integrals)
    (1, 1, [(O.QOI_MEASURE, None)], [(O.QOI_MEASURE, ALL_SIDES, None)]),
    (2, 1, [(O.QOI_POSITION, [1.0, -2.0, 0.5]), (O.QOI_POLY_TEST, None)], [(O.QOI_POLY_TEST, [1, 3, 6], None)]),
    (1, 3, [(O.QOI_FIELD, [1.0, 2.0, -1.0]), (O.QOI_POLY_TEST, None)],
     [(O.QOI_NORMAL_FIELD, ALL_SIDES, None), (O.QOI_POLY_TEST, [2, 5], None)]),
    (2, 3, [(O.QOI_NEOHOOKEAN_ENERGY, [5.0, 0.25])], [(O.QOI_NORMAL_FIELD, [6], None), (O.QOI_FIELD, [4], [0, 0, 1])]),
    (2, 3, [(O.QOI_POLY_TEST, None)], []),
    (1, 1, [], [(O.QOI_POLY_TEST, ALL_SIDES, None)]),
]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("shape_amp", [0.0, 0.02])
def test_qoi_parity(cuda, case, shape_amp):
    import serac_gb300 as sg

    p, c, domain, faces = CASES[case]
    orc, q = _qoi_pair(p, c, domain, faces, shape_amp=shape_amp)
    rng = np.random.default_rng(17 + case)
    amp = 0.01 if any(k == O.QOI_NEOHOOKEAN_ENERGY for k, _ in domain) else 0.1
    u = rng.standard_normal(orc.ndofs) * amp
    du = rng.standard_normal(orc.ndofs)
    ut, dut = torch.tensor(u, device=cuda), torch.tensor(du, device=cuda)
    value, grad = orc.evaluate(u)
    assert abs(q(0.0, ut) - value) <= 1e-12 * max(1.0, abs(value))
    v, dQ = q(0.0, sg.differentiate_wrt(ut))
    assert v == q(0.0, ut)
    g = sg.assemble(dQ).cpu().numpy()
    assert rel(g, grad) <= 1e-12
    act = dQ(dut)
    assert abs(act - grad @ du) <= 1e-12 * max(1.0, np.abs(grad).sum() * np.abs(du).max())
    # value written by the gradient call equals the evaluation
    val_t = torch.empty(1, dtype=torch.float64, device=cuda)
    q.gradient(0.0, ut, value=val_t)
    assert abs(float(val_t.item()) - v) <= 1e-14 * max(1.0, abs(v))


def test_qoi_exact_integrals(cuda):
    import serac_gb300 as sg

    m = mesh(4, 3, 2, perturb=0.2, seed=3)
    M = sg.Mesh.structured_hex(4, 3, 2, m.vertices)
    for p in (1, 2):
        u = torch.zeros(m.num_nodes(p), dtype=torch.float64, device=cuda)
        vol = sg.QoI(M, sg.H1(p, 1))
        vol.AddDomainIntegral(sg.QOI_MEASURE)
        assert abs(vol(0.0, u) - 1.0) <= 1e-12
        xm = sg.QoI(M, sg.H1(p, 1))
        xm.AddDomainIntegral(sg.QOI_POSITION, [1.0, 0.0, 0.0])
        assert abs(xm(0.0, u) - 0.5) <= 1e-12
        area = sg.QoI(M, sg.H1(p, 1))
        area.AddBoundaryIntegral(sg.QOI_MEASURE, ALL_SIDES)
        assert abs(area(0.0, u) - 6.0) <= 1e-12


@pytest.mark.parametrize("p", [1, 2])
def test_energy_gradient_equals_residual(cuda, p):
    """dW/du of the Neo-Hookean energy QoI is the Neo-Hookean residual (two
    independent kernels: AD of the energy vs the stress q-function)."""
    import serac_gb300 as sg

    m = mesh(4, 3, 3, perturb=0.1, seed=8)
    M = sg.Mesh.structured_hex(4, 3, 3, m.vertices)
    q = sg.QoI(M, sg.H1(p, 3))
    q.AddDomainIntegral(sg.QOI_NEOHOOKEAN_ENERGY, [5.0, 0.25])
    f = sg.Functional(M, sg.H1(p, 3))
    f.AddDomainIntegral(sg.NEOHOOKEAN, [5.0, 0.25])
    u = torch.tensor(np.random.default_rng(2).standard_normal(f.ndofs) * 0.01, device=cuda)
    g = q.gradient(0.0, u)
    r = f.residual(0.0, u)
    assert rel(g.cpu().numpy(), r.cpu().numpy()) <= 1e-12


TCASES = [
    # (material, p, boundary integral or None)
    (O.MAT_NONLINEAR_HEAT, 2, None),
    (O.MAT_NONLINEAR_HEAT, 1, (O.BMAT_HEAT_FLUX, (1, 3), [0.3, 0.7, 1.1])),
    (O.MAT_THERMAL_TEST, 2, None),
    (O.MAT_ELASTIC_TEST, 1, None),
    (O.MAT_NEOHOOKEAN, 2, (O.BMAT_PRESSURE, (1, 2, 3, 4, 5, 6), [0.7])),
    (O.MAT_J2, 2, None),
    (O.MAT_HEAT, 1, None),
]


@pytest.mark.parametrize("case", range(len(TCASES)))
def test_jvp_transpose_parity(cuda, case):
    import serac_gb300 as sg

    mat, p, bnd = TCASES[case]
    m = mesh(3, 2, 2, perturb=0.1, seed=5)
    c = O.COMPONENTS[mat]
    orc = O.OracleFunctional(m, p, c)
    f = sg.Functional(sg.Mesh.structured_hex(3, 2, 2, m.vertices), sg.H1(p, c))
    orc.add_domain_integral(mat, PARAMS[mat])
    f.AddDomainIntegral(mat, PARAMS[mat])
    if bnd is not None:
        orc.add_boundary_integral(*bnd)
        f.AddBoundaryIntegral(*bnd)
    rng = np.random.default_rng(23 + case)
    u = rng.standard_normal(orc.ndofs) * (0.02 if c == 3 else 0.3)
    w = rng.standard_normal(orc.ndofs)
    ut, wt = torch.tensor(u, device=cuda), torch.tensor(w, device=cuda)
    _, g = f(0.0, sg.differentiate_wrt(ut))
    ref = orc.jvp_transpose(u, w)
    assert rel(g.MultTranspose(wt).cpu().numpy(), ref) <= 1e-12
    assert rel(g.MultTranspose(wt.float()).double().cpu().numpy(), ref) <= 1e-5


def test_jvp_transpose_requires_stored_tangent(cuda):
    import serac_gb300 as sg
    from serac_gb300._lib import SfxError

    m = mesh(2, 2, 2)
    f = sg.Functional(sg.Mesh.structured_hex(2, 2, 2, m.vertices), sg.H1(1, 1))
    f.AddDomainIntegral(sg.HEAT, PARAMS[O.MAT_HEAT])
    f.set_jvp_mode(f.RECOMPUTE)
    u = torch.zeros(f.ndofs, dtype=torch.float64, device=cuda)
    _, g = f(0.0, sg.differentiate_wrt(u))
    with pytest.raises(SfxError):
        g.MultTranspose(u)


def test_adjoint_identity_full_size(cuda):
    """<w, J v> = <J^T w, v> on the 32^3 Q2 Neo-Hookean problem with follower
    pressure (non-symmetric boundary term), in FP64 and FP32."""
    import serac_gb300 as sg

    n = 32
    V = sg.box_vertices(n, n, n, perturb=0.1, seed=1)
    f = sg.Functional(sg.Mesh.structured_hex(n, n, n, V), sg.H1(2, 3))
    f.AddDomainIntegral(sg.NEOHOOKEAN, [5.0, 0.25])
    f.AddBoundaryIntegral(sg.PRESSURE, [6], [0.05])
    # smooth compression along z plus small noise (det F stays near 1)
    X = f.mesh.node_coordinates(2)
    nn = X.shape[0]
    u_h = np.zeros(3 * nn)
    u_h[2 * nn:] = -0.005 * X[:, 2]
    u_h += 1e-4 * np.random.default_rng(3).standard_normal(3 * nn)
    u = torch.tensor(u_h, device=cuda)
    gen = torch.Generator(device=cuda).manual_seed(3)
    v = torch.randn(f.ndofs, dtype=torch.float64, device=cuda, generator=gen)
    w = torch.randn(f.ndofs, dtype=torch.float64, device=cuda, generator=gen)
    _, g = f(0.0, sg.differentiate_wrt(u))
    Jv = g(v)
    assert bool(torch.isfinite(Jv).all())
    scale = float(torch.linalg.norm(w) * torch.linalg.norm(Jv))  # bound of the rounding of either dot
    lhs = float(torch.dot(w, Jv))
    rhs = float(torch.dot(g.MultTranspose(w), v))
    assert abs(lhs - rhs) <= 1e-13 * scale
    lhs32 = float(torch.dot(w, g(v.float()).double()))
    rhs32 = float(torch.dot(g.MultTranspose(w.float()).double(), v))
    assert abs(lhs32 - rhs32) <= 1e-5 * scale
    # the boundary term makes J non-symmetric: J^T w differs from J w
    assert rel(g.MultTranspose(w).cpu().numpy(), g(w).cpu().numpy()) > 1e-8


@pytest.mark.parametrize("krylov", ["gmres", "fgmres_mixed"])
def test_adjoint_solve(cuda, krylov):
    """lambda = J^-T b on the free vdofs for a non-symmetric operator,
    against a sparse direct solve of the eliminated transposed matrix."""
    import scipy.sparse.linalg as spla

    import serac_gb300 as sg

    m = mesh(4, 3, 3, perturb=0.1, seed=12)
    p = 2
    orc = O.OracleFunctional(m, p, 1)
    orc.add_domain_integral(O.MAT_NONLINEAR_HEAT, PARAMS[O.MAT_NONLINEAR_HEAT])
    f = sg.Functional(sg.Mesh.structured_hex(4, 3, 3, m.vertices), sg.H1(p, 1))
    f.AddDomainIntegral(sg.NONLINEAR_HEAT, PARAMS[O.MAT_NONLINEAR_HEAT])
    ess = m.boundary_nodes(p, [5])
    rng = np.random.default_rng(13)
    u = rng.standard_normal(orc.ndofs) * 0.3
    b = rng.standard_normal(orc.ndofs)
    if krylov == "gmres":
        opt = sg.SolverOptions.defaults(krylov=sg.GMRES, precond=sg.JACOBI, krylov_rel_tol=1e-12, krylov_abs_tol=0.0)
    else:
        opt = sg.SolverOptions.defaults(krylov=sg.FGMRES, precond=sg.JACOBI_CHEBYSHEV, mixed_precision=1,
                                        krylov_rel_tol=1e-12, krylov_abs_tol=0.0)
    s = sg.NewtonSolver(f, opt)
    s.set_essential(ess)
    lam = s.solve_adjoint(0.0, torch.tensor(u, device=cuda), torch.tensor(b, device=cuda)).cpu().numpy()
    A = O.eliminate_dirichlet(orc.assemble(u), ess)
    bb = b.copy()
    bb[ess] = 0.0
    ref = spla.spsolve(A.T.tocsc(), bb)
    assert rel(lam, ref) <= 1e-9
    assert np.all(lam[ess] == 0.0)
    # the forward solve differs (J is not symmetric)
    x = s.solve_linear(0.0, torch.tensor(u, device=cuda), torch.tensor(b, device=cuda)).cpu().numpy()
    assert rel(x, ref) > 1e-6
