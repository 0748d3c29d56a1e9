"""Shape displacement in the oracle (serac's ShapeAwareFunctional,
shape_aware_functional.hpp:45-172), pinned on the CPU: a shape field that is
the trilinear interpolant of a vertex displacement d describes exactly the
mesh whose vertices moved by d, so the shape-aware residual, Jacobian action
and boundary terms must equal the plain ones on that moved mesh — computed by
the reference's own element kernels (oracle/_ref) when they are built, and by
the restatement otherwise.  p = 0 must reproduce the plain functional."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.problems import PARAMS, rel


def _ref_available():
    return O.ref_lib() is not None


def _pair(mat, c, n=3, p=2, bmat=None):
    V = O.box_vertices(n, n, n, 0.1, 4)
    rng = np.random.default_rng(9)
    d = rng.uniform(-0.08, 0.08, V.shape) / n
    use_ref = _ref_available()
    base = O.StructuredHexMesh(n, n, n, V)
    moved = O.StructuredHexMesh(n, n, n, V + d)
    f_shape = O.OracleFunctional(base, p, c)
    f_moved = O.OracleFunctional(moved, p, c, use_ref=use_ref)
    for f in (f_shape, f_moved):
        f.add_domain_integral(mat, PARAMS[mat])
        if bmat is not None:
            f.add_boundary_integral(bmat, [3, 6], {O.BMAT_TRACTION: [0.3, -0.2, 0.5, 0.1, 0.0, -0.2],
                                                  O.BMAT_PRESSURE: [0.7]}[bmat])
    shape = (moved.node_coordinates(p) - base.node_coordinates(p)).T.ravel()
    f_shape.set_shape(shape)
    return f_shape, f_moved, rng


@pytest.mark.parametrize("mat,c", [(O.MAT_HEAT, 1), (O.MAT_NEOHOOKEAN, 3), (O.MAT_ELASTIC_TEST, 3)])
def test_trilinear_shape_equals_moved_mesh(mat, c):
    f_shape, f_moved, rng = _pair(mat, c)
    u = rng.standard_normal(f_shape.ndofs) * (0.02 if c == 3 else 0.3)
    du = rng.standard_normal(f_shape.ndofs)
    assert rel(f_shape.residual(u), f_moved.residual(u)) <= 1e-12
    assert rel(f_shape.jvp(u, du), f_moved.jvp(u, du)) <= 1e-12


@pytest.mark.parametrize("bmat", [O.BMAT_TRACTION, O.BMAT_PRESSURE])
def test_trilinear_shape_boundary_equals_moved_mesh(bmat):
    f_shape, f_moved, rng = _pair(O.MAT_NEOHOOKEAN, 3, bmat=bmat)
    u = rng.standard_normal(f_shape.ndofs) * 0.02
    du = rng.standard_normal(f_shape.ndofs)
    assert rel(f_shape.residual(u), f_moved.residual(u)) <= 1e-12
    assert rel(f_shape.jvp(u, du), f_moved.jvp(u, du)) <= 1e-12


def test_zero_shape_is_the_plain_functional():
    n, p = 2, 2
    m = O.StructuredHexMesh(n, n, n, O.box_vertices(n, n, n, 0.1, 1))
    f = O.OracleFunctional(m, p, 3)
    f.add_domain_integral(O.MAT_NEOHOOKEAN, PARAMS[O.MAT_NEOHOOKEAN])
    u = np.random.default_rng(0).standard_normal(f.ndofs) * 0.02
    r0 = f.residual(u)
    f.set_shape(np.zeros(3 * f.nnodes))
    assert rel(f.residual(u), r0) <= 1e-15
    f.set_shape(None)
    assert np.array_equal(f.residual(u), r0)
