"""The oracle on imported element tables (general hexahedral meshes): a
structured mesh rewritten with random node ids, random element order and a
random proper rotation of every element's local frame gives the same
residual, Jacobian action and CSR matrix (permuted), boundary integrals
included.  This pins the table path of the oracle against its structured
path, which is pinned against the reference kernels."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from tests.problems import PARAMS, ScrambledTable, cube_rotations, mesh, rel


def test_cube_rotations():
    R = cube_rotations()
    assert len(R) == 24
    assert len({r.tobytes() for r in R}) == 24


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("mat", [O.MAT_HEAT, O.MAT_NEOHOOKEAN, O.MAT_THERMAL_TEST])
def test_scrambled_table_matches_structured(p, mat):
    m = mesh(3, 2, 2, perturb=0.1, seed=5)
    c = O.COMPONENTS[mat]
    st = ScrambledTable(m, p, seed=3)
    tm = O.TableHexMesh(p, st.table, st.corners, st.nn)
    a = O.OracleFunctional(m, p, c)
    b = O.OracleFunctional(tm, p, c)
    a.add_domain_integral(mat, PARAMS[mat])
    b.add_domain_integral(mat, PARAMS[mat])
    bm, bp = (O.BMAT_HEAT_FLUX, [0.3, 0.7, 1.1]) if c == 1 else (O.BMAT_PRESSURE, [0.7])
    a.add_boundary_integral(bm, [1, 3, 6], bp)
    b.add_boundary_integral(bm, st.faces_of_sides([1, 3, 6]), bp)
    rng = np.random.default_rng(1)
    u = rng.standard_normal(a.ndofs) * 0.02
    du = rng.standard_normal(a.ndofs)
    un, dun = st.to_new(u, c), st.to_new(du, c)
    assert rel(b.residual(un), st.to_new(a.residual(u), c)) <= 1e-13
    assert rel(b.jvp(un, dun), st.to_new(a.jvp(u, du), c)) <= 1e-13
    P = st.vdof_perm(c)
    Pm = sp.csr_matrix((np.ones(len(P)), (P, np.arange(len(P)))), shape=(len(P), len(P)))
    A, B = a.assemble(u), b.assemble(un)
    assert abs(Pm @ A @ Pm.T - B).max() <= 1e-13 * abs(A).max()
