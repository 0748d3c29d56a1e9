"""The oracle (CPU restatement) against serac's own numbers.

* golden fixtures generated from serac's element kernels (tests/golden/)
* serac's element kernels compiled from the reference sources, where present
* property checks of serac's own test suite: matrix-free vs assembled Jv and
  finite-difference convergence (check_gradient.hpp:16-90), patch test
  (solid_statics_patch.cpp: affine fields give zero interior residual)
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.problems import PARAMS, fields, mesh, rel

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _domain_fixtures():
    return sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz")) if "material" in np.load(f).files)


def _boundary_fixtures():
    return sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz")) if "bmaterial" in np.load(f).files)


def test_fixtures_present():
    assert len(_domain_fixtures()) >= 10 and len(_boundary_fixtures()) >= 3


@pytest.mark.parametrize("path", _domain_fixtures(), ids=lambda p: os.path.basename(p))
def test_oracle_matches_golden_domain(path):
    g = np.load(path)
    mat, p = int(g["material"]), int(g["order"])
    m = mesh(*g["dims"], perturb=float(g["perturb"]), seed=int(g["seed"]))
    f = O.OracleFunctional(m, p, O.COMPONENTS[mat])
    f.add_domain_integral(mat, PARAMS[mat])
    u, du = fields(f.ndofs, mat, seed=int(g["seed"]))
    if mat == O.MAT_J2:
        assert rel(f.residual(u, update_state=True), g["residual_commit"]) <= 1e-13
        assert np.max(np.abs(f.state - g["state"])) <= 1e-13 * max(1.0, np.abs(g["state"]).max())
        u = 1.5 * u
    assert rel(f.residual(u), g["residual"]) <= 1e-13
    assert rel(f.jvp(u, du), g["jvp"]) <= 1e-13
    A = f.assemble(u)
    assert np.array_equal(A.indptr, g["csr_row_ptr"])
    assert np.array_equal(A.indices, g["csr_col"])
    assert rel(A.data, g["csr_val"]) <= 1e-13


@pytest.mark.parametrize("path", _boundary_fixtures(), ids=lambda p: os.path.basename(p))
def test_oracle_matches_golden_boundary(path):
    g = np.load(path)
    bmat, p = int(g["bmaterial"]), int(g["order"])
    m = mesh(*g["dims"], perturb=0.1, seed=int(g["seed"]))
    f = O.OracleFunctional(m, p, O.BCOMPONENTS[bmat])
    f.add_boundary_integral(bmat, [int(s) for s in g["sides"]], g["params"])
    assert rel(f.residual(g["u"]), g["residual"]) <= 1e-13
    assert rel(f.jvp(g["u"], g["du"]), g["jvp"]) <= 1e-13


@pytest.mark.skipif(O.ref_lib() is None, reason="reference sources not present (checker not built)")
@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("mat", sorted(PARAMS))
def test_oracle_element_kernels_match_reference(mat, p):
    rng = np.random.default_rng(100 * mat + p)
    m = mesh(3, 2, 2, perturb=0.15, seed=p)
    Xq, Jq = O.geometric_factors(m.elem_coords(), p + 1, use_ref=True)
    Xo, Jo = O.geometric_factors(m.elem_coords(), p + 1)
    assert np.abs(Xq - Xo).max() <= 1e-15 and np.abs(Jq - Jo).max() <= 1e-14
    c = O.COMPONENTS[mat]
    nd = (p + 1) ** 3 * c
    amp = 0.01 if mat in (O.MAT_NEOHOOKEAN, O.MAT_J2) else 0.1
    uE = rng.standard_normal((m.ne, nd)) * amp
    duE = rng.standard_normal((m.ne, nd))
    tol = 1e-14 if p < 3 else 1e-13
    for mode in (0, 1, 2):
        a = O.element_kernel(mat, p, mode, uE, Xq, Jq, PARAMS[mat], duE)
        b = O.element_kernel(mat, p, mode, uE, Xq, Jq, PARAMS[mat], duE, use_ref=True)
        assert rel(a, b) <= tol, (mode, rel(a, b))


@pytest.mark.parametrize("mat", [O.MAT_NEOHOOKEAN, O.MAT_NONLINEAR_HEAT, O.MAT_ELASTIC_TEST])
def test_check_gradient(mat):
    """check_gradient.hpp:16-90: matrix-free Jv equals the assembled matrix
    times v, and the finite-difference errors shrink at first / second order."""
    m = mesh(3, 2, 2)
    f = O.OracleFunctional(m, 2, O.COMPONENTS[mat])
    f.add_domain_integral(mat, PARAMS[mat])
    u, _ = fields(f.ndofs, mat, seed=1)
    dU = np.random.default_rng(42).uniform(0, 1, f.ndofs)
    jv = f.jvp(u, dU)
    A = f.assemble(u)
    assert rel(A @ dU, jv) <= 1e-12
    eps = 1e-4
    fv = [f.residual(u + (i - 2) * eps * dU) for i in range(5)]
    den = np.linalg.norm(jv)
    e1 = np.linalg.norm((fv[4] - fv[2]) / (2 * eps) - jv) / den
    e2 = np.linalg.norm((fv[3] - fv[2]) / eps - jv) / den
    e3 = np.linalg.norm((fv[4] - fv[0]) / (4 * eps) - jv) / den
    e4 = np.linalg.norm((fv[3] - fv[1]) / (2 * eps) - jv) / den
    assert abs(e1 / e2 - 2.0) < 0.1 or min(e1, e2) < 1e-9
    assert abs(e3 / e4 - 4.0) < 0.1 or min(e3, e4) < 1e-9


@pytest.mark.parametrize("p", [1, 2])
def test_patch_test_neohookean(p):
    """An affine displacement gives a uniform stress, so the residual vanishes
    at every node away from the boundary (solid_statics_patch.cpp)."""
    m = mesh(3, 3, 3, perturb=0.2, seed=3)
    f = O.OracleFunctional(m, p, 3)
    f.add_domain_integral(O.MAT_NEOHOOKEAN, PARAMS[O.MAT_NEOHOOKEAN])
    N = f.nnodes
    Np = (p * 3 + 1)
    idx = np.arange(N)
    I, J, K = idx % Np, (idx // Np) % Np, idx // (Np * Np)
    # nodal coordinates by the trilinear map are not needed: an affine field in
    # the reference grid index space is affine in X only on an unperturbed
    # mesh, so use an unperturbed mesh for the field and perturbed geometry off
    m0 = mesh(3, 3, 3, perturb=0.0)
    f0 = O.OracleFunctional(m0, p, 3)
    f0.add_domain_integral(O.MAT_NEOHOOKEAN, PARAMS[O.MAT_NEOHOOKEAN])
    X = np.stack([I, J, K], axis=1) / (p * 3.0)
    Gm = np.array([[0.01, 0.02, -0.01], [0.0, -0.015, 0.01], [0.005, 0.0, 0.02]])
    u = (X @ Gm.T).T.ravel()
    r = f0.residual(u).reshape(3, N)
    interior = (I > 0) & (I < Np - 1) & (J > 0) & (J < Np - 1) & (K > 0) & (K < Np - 1)
    assert np.abs(r[:, interior]).max() <= 1e-14
    assert np.abs(r[:, ~interior]).max() > 1e-6
    del f


def test_cg_solves_config1_small():
    """Linear steady heat, Dirichlet x=0: Jacobi CG reaches 1e-10."""
    n = 4
    m = mesh(n, n, n, perturb=0.0)
    f = O.OracleFunctional(m, 2, 1)
    f.add_domain_integral(O.MAT_HEAT, [1.0, 1.0])
    u0 = np.zeros(f.ndofs)
    b = -f.residual(u0)
    ess = m.boundary_nodes(2, [5])
    b[ess] = 0.0
    A = O.eliminate_dirichlet(f.assemble(u0), ess)
    x, it, res = O.cg(lambda v: A @ v, b, A.diagonal(), rtol=1e-10)
    assert res < 1e-10
    # solution is positive away from x = 0 and grows with x
    assert x[ess].max() == 0.0 and x.max() > 0.0
