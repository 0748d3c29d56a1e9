"""Forms built from imported element tables (sfx_form_create_from_table, the
mfem element-dof table path) on the GPU: a structured mesh rewritten with
random node ids, random element order and randomly rotated element frames
gives the structured form's residual, Jacobian actions (FP64, FP32,
transposed), diagonal, CSR matrix, boundary integrals, quantities of
interest and Newton solution, permuted; and the table form matches the
oracle's table path directly."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import oracle as O
from tests.problems import PARAMS, ScrambledTable, mesh, rel

pytestmark = pytest.mark.gpu

DIMS = (3, 2, 2)
CASES = [
    (O.MAT_HEAT, 1, (O.BMAT_HEAT_FLUX, [1, 3, 6], [0.3, 0.7, 1.1])),
    (O.MAT_NONLINEAR_HEAT, 2, (O.BMAT_HEAT_FLUX, [2, 5], [0.1, -0.2, 0.5])),
    (O.MAT_THERMAL_TEST, 2, None),
    (O.MAT_NEOHOOKEAN, 2, (O.BMAT_PRESSURE, [3, 6], [0.7])),
    (O.MAT_NEOHOOKEAN, 1, (O.BMAT_TRACTION, [4], [0.1, 0.2, 0.3, 0.5, -0.4, 0.2])),
    (O.MAT_J2, 2, None),
]


def _forms(mat, p, bnd, seed=3):
    import serac_gb300 as sg

    m = mesh(*DIMS, perturb=0.1, seed=5)
    st = ScrambledTable(m, p, seed=seed)
    c = O.COMPONENTS[mat]
    fs = sg.Functional(sg.Mesh.structured_hex(*DIMS, m.vertices), sg.H1(p, c))
    ft = sg.Functional(sg.TableMesh(p, st.table, st.corners, st.nn), sg.H1(p, c))
    fs.AddDomainIntegral(mat, PARAMS[mat])
    ft.AddDomainIntegral(mat, PARAMS[mat])
    if bnd is not None:
        bmat, sides, bp = bnd
        fs.AddBoundaryIntegral(bmat, sides, bp)
        ft.AddBoundaryIntegral(bmat, params=bp, faces=st.faces_of_sides(sides))
    return m, st, fs, ft, c


def _csr(f):
    import serac_gb300 as sg

    row_ptr, col, val = sg.assemble(f.gradient)
    n = f.ndofs
    return sp.csr_matrix((val.cpu().numpy(), col.cpu().numpy().astype(np.int64), row_ptr.cpu().numpy()), shape=(n, n))


@pytest.mark.parametrize("case", range(len(CASES)))
def test_table_form_matches_structured(cuda, case):
    import serac_gb300 as sg

    mat, p, bnd = CASES[case]
    m, st, fs, ft, c = _forms(mat, p, bnd)
    rng = np.random.default_rng(90 + case)
    u = rng.standard_normal(fs.ndofs) * (0.02 if c == 3 else 0.3)
    du = rng.standard_normal(fs.ndofs)
    P = torch.tensor(st.vdof_perm(c), device=cuda)

    def new(x):
        out = torch.empty_like(x)
        out[P] = x
        return out

    us, dus = torch.tensor(u, device=cuda), torch.tensor(du, device=cuda)
    ut, dut = new(us), new(dus)
    assert rel(ft.residual(0.0, ut).cpu().numpy(), new(fs.residual(0.0, us)).cpu().numpy()) <= 1e-12
    rs, gs = fs(0.0, sg.differentiate_wrt(us))
    rt, gt = ft(0.0, sg.differentiate_wrt(ut))
    assert rel(rt.cpu().numpy(), new(rs).cpu().numpy()) <= 1e-12
    assert rel(gt(dut).cpu().numpy(), new(gs(dus)).cpu().numpy()) <= 1e-12
    ref32 = new(gs(dus)).cpu().numpy()
    assert rel(gt(dut.float()).double().cpu().numpy(), ref32) <= 1e-5
    assert rel(gt.MultTranspose(dut).cpu().numpy(), new(gs.MultTranspose(dus)).cpu().numpy()) <= 1e-12
    assert rel(ft.assemble_diagonal().cpu().numpy(), new(fs.assemble_diagonal()).cpu().numpy()) <= 1e-12
    A, B = _csr(fs), _csr(ft)
    Pn = st.vdof_perm(c)
    Pm = sp.csr_matrix((np.ones(len(Pn)), (Pn, np.arange(len(Pn)))), shape=(len(Pn), len(Pn)))
    assert B.nnz == A.nnz
    assert abs(Pm @ A @ Pm.T - B).max() <= 1e-12 * abs(A).max()
    # columns sorted within every row
    for r in range(0, B.shape[0], max(1, B.shape[0] // 50)):
        cols = B.indices[B.indptr[r]:B.indptr[r + 1]]
        assert np.all(np.diff(cols) > 0)


@pytest.mark.parametrize("case", [0, 3])
def test_table_form_matches_oracle(cuda, case):
    import serac_gb300 as sg

    mat, p, bnd = CASES[case]
    m, st, _, ft, c = _forms(mat, p, bnd, seed=7)
    tm = O.TableHexMesh(p, st.table, st.corners, st.nn)
    orc = O.OracleFunctional(tm, p, c)
    orc.add_domain_integral(mat, PARAMS[mat])
    if bnd is not None:
        orc.add_boundary_integral(bnd[0], st.faces_of_sides(bnd[1]), bnd[2])
    rng = np.random.default_rng(95 + case)
    u = rng.standard_normal(ft.ndofs) * (0.02 if c == 3 else 0.3)
    du = rng.standard_normal(ft.ndofs)
    ut = torch.tensor(u, device=cuda)
    assert rel(ft.residual(0.0, ut).cpu().numpy(), orc.residual(u)) <= 1e-12
    _, g = ft(0.0, sg.differentiate_wrt(ut))
    assert rel(g(torch.tensor(du, device=cuda)).cpu().numpy(), orc.jvp(u, du)) <= 1e-12
    A = orc.assemble(u)
    B = _csr(ft)
    assert abs(A - B).max() <= 1e-12 * abs(A).max()


def test_table_newton_matches_structured(cuda):
    """Neo-Hookean under a follower pressure, clamped on z = 0: Newton on the
    scrambled table converges to the structured solution (permuted)."""
    import serac_gb300 as sg

    mat, p, bnd = CASES[3]
    m, st, fs, ft, c = _forms(mat, p, (O.BMAT_PRESSURE, [6], [0.02]))
    ess_nodes = m.boundary_nodes(p, [1])
    ess_s = np.concatenate([k * st.nn + ess_nodes for k in range(3)])
    ess_t = st.vdof_perm(3)[ess_s]
    opts = sg.SolverOptions.defaults(newton_rel_tol=1e-10, newton_abs_tol=0.0, krylov_rel_tol=1e-10,
                                     krylov_abs_tol=0.0)
    sol = []
    for f, ess in ((fs, ess_s), (ft, ess_t)):
        s = sg.NewtonSolver(f, opts)
        s.set_essential(ess)
        u = torch.zeros(f.ndofs, dtype=torch.float64, device=cuda)
        s.solve(0.0, u)
        sol.append(u.cpu().numpy())
    assert np.linalg.norm(sol[0]) > 0
    assert rel(sol[1], st.to_new(sol[0], 3)) <= 1e-8


def test_table_qoi_matches_structured(cuda):
    import serac_gb300 as sg

    p, c = 2, 3
    m = mesh(*DIMS, perturb=0.1, seed=5)
    st = ScrambledTable(m, p, seed=11)
    qs = sg.QoI(sg.Mesh.structured_hex(*DIMS, m.vertices), sg.H1(p, c))
    qt = sg.QoI(sg.TableMesh(p, st.table, st.corners, st.nn), sg.H1(p, c))
    for q in (qs, qt):
        q.AddDomainIntegral(sg.QOI_NEOHOOKEAN_ENERGY, [5.0, 0.25])
    qs.AddBoundaryIntegral(sg.QOI_NORMAL_FIELD, [2, 6])
    qt.AddBoundaryIntegral(sg.QOI_NORMAL_FIELD, faces=st.faces_of_sides([2, 6]))
    u = np.random.default_rng(4).standard_normal(st.nn * c) * 0.01
    us = torch.tensor(u, device=cuda)
    ut = torch.tensor(st.to_new(u, c), device=cuda)
    vs, vt = qs(0.0, us), qt(0.0, ut)
    assert abs(vs - vt) <= 1e-12 * abs(vs)
    assert rel(qt.gradient(0.0, ut).cpu().numpy(), st.to_new(qs.gradient(0.0, us).cpu().numpy(), c)) <= 1e-12


def test_table_form_rejects_side_masks(cuda):
    import serac_gb300 as sg
    from serac_gb300._lib import SfxError

    m = mesh(2, 2, 2)
    st = ScrambledTable(m, 1, seed=1)
    f = sg.Functional(sg.TableMesh(1, st.table, st.corners, st.nn), sg.H1(1, 1))
    with pytest.raises(SfxError):
        f.AddBoundaryIntegral(sg.HEAT_FLUX, [1], [0.1, 0.0, 0.0])
    bad = st.table.copy()
    bad[0, 0] = st.nn + 5
    with pytest.raises(SfxError):
        sg.Functional(sg.TableMesh(1, bad, st.corners, st.nn), sg.H1(1, 1))
