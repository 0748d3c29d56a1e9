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


@pytest.mark.parametrize("p", [1, 2])
def test_every_frame_rotation(p):
    """All 24 proper rotations of one element's local frame (the other element
    keeps its frame) leave the residual, Jacobian action and boundary
    integrals unchanged."""
    from tests.problems import _SIDE_OF, _DIR_OF, _local_map

    m = mesh(2, 1, 1, perturb=0.0)
    V = m.vertices.copy()
    V[:, 2] += 0.05 * V[:, 0] * V[:, 1]  # not a brick
    m = O.StructuredHexMesh(2, 1, 1, V)
    n = p + 1
    conn = m.elem_nodes(p)
    Xe = m.elem_coords()
    ref = O.OracleFunctional(m, p, 3)
    ref.add_domain_integral(O.MAT_NEOHOOKEAN, PARAMS[O.MAT_NEOHOOKEAN])
    ref.add_boundary_integral(O.BMAT_PRESSURE, [3, 6], [0.7])
    rng = np.random.default_rng(2)
    u = rng.standard_normal(ref.ndofs) * 0.02
    du = rng.standard_normal(ref.ndofs)
    r0, j0 = ref.residual(u), ref.jvp(u, du)
    for R in cube_rotations():
        table = conn.copy()
        corners = Xe.transpose(0, 2, 1).copy()
        table[1] = conn[1][_local_map(R, n)]
        corners[1] = Xe[1].T[_local_map(R, 2)]
        # faces of box sides 3 (x = 1, element 1 only) and 6 (z = 1, both elements)
        elems, sides = [], []
        for e, s in ((1, 3), (0, 6), (1, 6)):
            ax, hi = _DIR_OF[s]
            d = np.zeros(3, dtype=np.int64)
            d[ax] = 1 if hi else -1
            if e == 1:
                d = R @ d
            axn = int(np.flatnonzero(d)[0])
            elems.append(e)
            sides.append(_SIDE_OF[(axn, 1 if d[axn] > 0 else 0)])
        tm = O.TableHexMesh(p, table, corners, m.num_nodes(p))
        f = O.OracleFunctional(tm, p, 3)
        f.add_domain_integral(O.MAT_NEOHOOKEAN, PARAMS[O.MAT_NEOHOOKEAN])
        f.add_boundary_integral(O.BMAT_PRESSURE, (np.array(elems), np.array(sides)), [0.7])
        assert rel(f.residual(u), r0) <= 1e-13
        assert rel(f.jvp(u, du), j0) <= 1e-13
