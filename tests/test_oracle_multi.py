"""The multi-field oracle (Functional<test(displacement, acceleration, dK,
dG)> with the parameterized Neo-Hookean integrand of SolidMechanics) against
serac's own kernels: the committed fixtures written from them
(tests/golden/param_neohookean_p*.npz, make_golden.py multi) and, where the
reference checker is built here, the kernels themselves on fresh inputs.
Residual, Jacobian action and element matrices with respect to each argument
(evaluation_kernel_impl / action_of_gradient_kernel / element_gradient_kernel
over four trial spaces, domain_integral_kernels.hpp:152-361), 1e-13."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden.make_golden import multi_fields
from tests.problems import mesh, rel

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "param_neohookean_p*.npz"))))
def test_multi_oracle_matches_golden(path):
    g = np.load(path)
    m = mesh(*[int(x) for x in g["dims"]], perturb=float(g["perturb"]), seed=int(g["seed"]))
    f = O.OracleMultiFunctional(m, int(g["order"]), g["params"])
    flds = multi_fields(f.nnodes, int(g["seed"]))
    assert rel(f.residual(flds), g["residual"]) <= 1e-13
    for w in range(4):
        assert rel(f.jvp(flds, w, g[f"dir{w}"]), g[f"jvp{w}"]) <= 1e-13, w
        assert rel(f.element_matrices(flds, w), g[f"ke{w}"]) <= 1e-13, w


@pytest.mark.skipif(O.ref_lib() is None, reason="reference checker not built here")
@pytest.mark.parametrize("p", [1, 2])
def test_multi_oracle_matches_reference_kernels(p):
    m = mesh(3, 2, 2, perturb=0.1, seed=40 + p)
    f = O.OracleMultiFunctional(m, p, [1.1, 4.0, 0.3])
    flds = multi_fields(f.nnodes, 50 + p)
    rng = np.random.default_rng(p)
    assert rel(f.residual(flds), f.residual(flds, use_ref=True)) <= 1e-13
    for w, c in enumerate(O.MULTI_COMPONENTS):
        d = rng.standard_normal(c * f.nnodes)
        assert rel(f.jvp(flds, w, d), f.jvp(flds, w, d, use_ref=True)) <= 1e-13, w
        assert rel(f.element_matrices(flds, w), f.element_matrices(flds, w, use_ref=True)) <= 1e-13, w


def test_multi_transpose_is_the_adjoint():
    """v . J_w d = (J_w^T v) . d for every argument, and J_w^T v assembled
    from the element matrices equals the restated transposed action."""
    m = mesh(2, 2, 2, perturb=0.1, seed=3)
    f = O.OracleMultiFunctional(m, 2, [1.0, 5.0, 0.25])
    flds = multi_fields(f.nnodes, 7)
    rng = np.random.default_rng(9)
    for w, c in enumerate(O.MULTI_COMPONENTS):
        d = rng.standard_normal(c * f.nnodes)
        v = rng.standard_normal(3 * f.nnodes)
        lhs = v @ f.jvp(flds, w, d)
        rhs = f.jvp_transpose(flds, w, v) @ d
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs), w


def test_multi_parameter_derivative_matches_finite_differences():
    m = mesh(2, 1, 2, perturb=0.1, seed=5)
    f = O.OracleMultiFunctional(m, 2, [1.0, 5.0, 0.25])
    flds = multi_fields(f.nnodes, 11)
    rng = np.random.default_rng(4)
    for w in (2, 3):
        d = rng.standard_normal(f.nnodes)
        h = 1e-6
        plus = [x.copy() for x in flds]
        minus = [x.copy() for x in flds]
        plus[w] += h * d
        minus[w] -= h * d
        fd = (f.residual(plus) - f.residual(minus)) / (2 * h)
        assert rel(f.jvp(flds, w, d), fd) <= 1e-7, w
