"""Quantity-of-interest oracle (Functional<double(...)>, functional_qoi.inl)
pinned on CPU: exact integrals of the perturbed unit cube (the reference's
functional_qoi.cpp checks measure, moments and areas to 1e-10), finite
differences of the gradient, the Neo-Hookean energy whose gradient must equal
the pinned Neo-Hookean residual, and the transposed Jacobian action."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.problems import mesh, rel

ALL_SIDES = [1, 2, 3, 4, 5, 6]


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("c", [1, 3])
def test_exact_integrals(p, c):
    m = mesh(3, 3, 2, perturb=0.2, seed=3)
    u = np.zeros(m.num_nodes(p) * c)
    cases = [
        (O.QOI_MEASURE, None, False, 1.0),            # volume
        (O.QOI_POSITION, [1.0, 0.0, 0.0], False, 0.5),  # x moment
        (O.QOI_POSITION, [0.0, 2.0, -1.0], False, 0.5),
        (O.QOI_MEASURE, None, True, 6.0),             # surface area
    ]
    for kind, params, boundary, exact in cases:
        q = O.OracleQoI(m, p, c)
        if boundary:
            q.add_boundary_integral(kind, ALL_SIDES, params)
        else:
            q.add_domain_integral(kind, params)
        assert abs(q.value(u) - exact) <= 1e-12


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("c", [1, 3])
def test_field_integral_of_affine_field(p, c):
    """w . u over the domain and the x = 1 side for an affine u, exactly."""
    m = mesh(3, 2, 2, perturb=0.15, seed=4)
    X = m.node_coordinates(p)
    a = np.array([0.3, -0.2, 0.5])
    comps = [1.0 + X @ a * (k + 1) for k in range(c)]
    u = np.concatenate(comps)
    w = np.arange(1, c + 1, dtype=np.float64)
    q = O.OracleQoI(m, p, c)
    q.add_domain_integral(O.QOI_FIELD, w)
    # integral of 1 + a.X over the unit cube = 1 + sum(a)/2
    exact = sum(w[k] * (1.0 + (k + 1) * a.sum() / 2) for k in range(c))
    assert abs(q.value(u) - exact) <= 1e-12
    qb = O.OracleQoI(m, p, c)
    qb.add_boundary_integral(O.QOI_FIELD, [3], w)  # x = 1: 1 + a0 + (a1 + a2)/2
    exact_b = sum(w[k] * (1.0 + (k + 1) * (a[0] + (a[1] + a[2]) / 2)) for k in range(c))
    assert abs(qb.value(u) - exact_b) <= 1e-12


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("c", [1, 3])
def test_gradient_finite_differences(p, c):
    m = mesh(3, 2, 2, perturb=0.15, seed=6)
    rng = np.random.default_rng(7)
    n = m.num_nodes(p) * c
    u = 0.1 * rng.standard_normal(n)
    du = rng.standard_normal(n)
    q = O.OracleQoI(m, p, c)
    q.add_domain_integral(O.QOI_POLY_TEST)
    q.add_boundary_integral(O.QOI_POLY_TEST, [1, 3, 6])
    if c == 3:
        q.add_boundary_integral(O.QOI_NORMAL_FIELD, [2, 4])
    g = q.gradient(u)
    h = 1e-6
    fd = (q.value(u + h * du) - q.value(u - h * du)) / (2 * h)
    assert abs(fd - g @ du) <= 1e-7 * abs(fd)


@pytest.mark.parametrize("p", [1, 2])
def test_neohookean_energy_gradient_is_residual(p):
    m = mesh(3, 2, 2, perturb=0.1, seed=8)
    rng = np.random.default_rng(9)
    u = 0.01 * rng.standard_normal(m.num_nodes(p) * 3)
    q = O.OracleQoI(m, p, 3)
    q.add_domain_integral(O.QOI_NEOHOOKEAN_ENERGY, [5.0, 0.25])
    f = O.OracleFunctional(m, p, 3)
    f.add_domain_integral(O.MAT_NEOHOOKEAN, [5.0, 0.25])
    assert rel(q.gradient(u), f.residual(u)) <= 1e-12


def test_jvp_transpose_is_the_adjoint():
    """<w, J v> = <J^T w, v> for a non-symmetric Jacobian (nonlinear heat)."""
    m = mesh(3, 2, 2, perturb=0.1, seed=10)
    f = O.OracleFunctional(m, 2, 1)
    f.add_domain_integral(O.MAT_NONLINEAR_HEAT, [1.0, 0.5, 1.0])
    rng = np.random.default_rng(11)
    u, v, w = (rng.standard_normal(f.ndofs) * s for s in (0.3, 1.0, 1.0))
    lhs = w @ f.jvp(u, v)
    rhs = f.jvp_transpose(u, w) @ v
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    A = f.assemble(u)
    assert abs(A - A.T).max() > 1e-3  # the operator really is non-symmetric


@pytest.mark.parametrize("p", [1, 2])
def test_shape_gradient_of_measures(p):
    """d(volume)/dp and d(area)/dp by finite differences: a uniform dilation
    p = eps X changes the volume at rate 3 V and the area at rate 2 A, a
    translation changes neither."""
    m = mesh(2, 2, 1, perturb=0.2, seed=3)
    X = m.node_coordinates(p)
    dil = np.concatenate([X[:, 0], X[:, 1], X[:, 2]])
    trans = np.concatenate([np.full(len(X), 0.3), np.full(len(X), -0.1), np.full(len(X), 0.2)])
    u = np.zeros(m.num_nodes(p))
    vol = O.OracleQoI(m, p, 1)
    vol.add_domain_integral(O.QOI_MEASURE)
    gv = vol.shape_gradient_fd(u)
    assert abs(gv @ dil - 3.0) <= 1e-7
    assert abs(gv @ trans) <= 1e-7
    area = O.OracleQoI(m, p, 1)
    area.add_boundary_integral(O.QOI_MEASURE, ALL_SIDES)
    ga = area.shape_gradient_fd(u)
    assert abs(ga @ dil - 12.0) <= 1e-7
    assert abs(ga @ trans) <= 1e-7


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("c", [1, 3])
def test_qoi_matches_reference_kernels(p, c):
    """Values and gradients against serac's own QoI element kernels
    (evaluation_kernel_impl / element_gradient_kernel with the QOI test space,
    compiled from the reference sources into oracle/_ref)."""
    if O.ref_lib() is None or not hasattr(O.ref_lib(), "ref_qoi"):
        pytest.skip("reference kernels not built here")
    m = mesh(3, 2, 2, perturb=0.15, seed=6)
    rng = np.random.default_rng(7)
    u = rng.standard_normal(m.num_nodes(p) * c) * (0.01 if c == 3 else 0.1)
    w = np.arange(1, c + 1, dtype=np.float64)
    q = O.OracleQoI(m, p, c)
    q.add_domain_integral(O.QOI_POLY_TEST)
    q.add_domain_integral(O.QOI_FIELD, w)
    q.add_boundary_integral(O.QOI_POLY_TEST, [1, 3, 6])
    q.add_boundary_integral(O.QOI_FIELD, [2], w)
    if c == 3:
        q.add_domain_integral(O.QOI_NEOHOOKEAN_ENERGY, [5.0, 0.25])
        q.add_boundary_integral(O.QOI_NORMAL_FIELD, [4, 5])
    v, g = q.evaluate(u)
    rv, rg = q.evaluate_reference(u)
    assert abs(v - rv) <= 1e-13 * abs(v)
    assert rel(g, rg) <= 1e-13


def _qoi_cases():
    import importlib.util
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.QOI_CASES


@pytest.mark.parametrize("case", _qoi_cases(), ids=lambda c: c[0])
def test_qoi_matches_golden_fixtures(case):
    """Values and gradients against the committed fixtures written from
    serac's own QOI element kernels (tests/golden/make_golden.py qoi)."""
    import os

    name, p, c, dims, domain, faces, seed = case
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"{name}.npz"))
    m = mesh(*dims, perturb=0.15, seed=seed)
    q = O.OracleQoI(m, p, c)
    for kind, params in domain:
        q.add_domain_integral(kind, params)
    for kind, sides, params in faces:
        q.add_boundary_integral(kind, sides, params)
    v, grad = q.evaluate(g["u"])
    assert abs(v - float(g["value"])) <= 1e-13 * abs(float(g["value"]))
    assert rel(grad, g["gradient"]) <= 1e-13
