"""The header-only C++ front-end (include/sfx/functional.hpp) with user-written
q-function objects compiled into a test library (tests/cpp/frontend_test.cu):
residual, linearised residual, FP64 / FP32 Jacobian action, diagonal and CSR
values against the oracle; quadrature-point state through QuadratureData."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests.problems import PARAMS, fields, mesh, rel

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpp", "frontend_test.cu")
LIB = os.path.join(HERE, "cpp", "libsfx_frontend_test.so")

_dp = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def felib():
    from serac_gb300 import _lib, build

    _lib.load()
    headers = [os.path.join(ROOT, "include", "sfx", f) for f in os.listdir(os.path.join(ROOT, "include", "sfx"))]
    newest = max([os.path.getmtime(SRC), os.path.getmtime(_lib.LIB_PATH)] + [os.path.getmtime(h) for h in headers])
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [build.nvcc(), *build.NVCC_FLAGS, "-shared", "-I", os.path.join(ROOT, "include"), "-o", LIB, SRC,
               "-L", os.path.dirname(_lib.LIB_PATH), "-lsfx_gb300", "-Xlinker", "-rpath=" + os.path.dirname(_lib.LIB_PATH)]
        subprocess.check_call(cmd)
    lib = ctypes.CDLL(LIB)
    return lib


def _p(a):
    return a.ctypes.data_as(_dp)


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("kind", ["thermal", "neohookean"])
def test_user_qfunction_matches_oracle(cuda, felib, kind, p):
    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=2)
    mat = O.MAT_THERMAL_TEST if kind == "thermal" else O.MAT_NEOHOOKEAN
    orc = O.OracleFunctional(m, p, O.COMPONENTS[mat])
    orc.add_domain_integral(mat, PARAMS[mat])
    u, du = fields(orc.ndofs, mat, seed=8)
    n = orc.ndofs
    outs = [np.zeros(n) for _ in range(5)]
    A = orc.assemble(u)
    csr = np.zeros(A.nnz)
    nnz = ctypes.c_int64()
    V = np.ascontiguousarray(m.vertices)
    if kind == "thermal":
        rc = felib.frontend_thermal(p, *dims, _p(V), _p(u), _p(du), *[_p(o) for o in outs], _p(csr), ctypes.byref(nnz))
    else:
        K, G = PARAMS[mat]
        rc = felib.frontend_neohookean(p, ctypes.c_double(K), ctypes.c_double(G), *dims, _p(V), _p(u), _p(du),
                                       *[_p(o) for o in outs], _p(csr), ctypes.byref(nnz))
    assert rc == 0
    r, r2, jv, jv32, diag = outs
    ref_r = orc.residual(u)
    assert rel(r, ref_r) <= 1e-12
    assert rel(r2, ref_r) <= 1e-12
    ref_jv = orc.jvp(u, du)
    assert rel(jv, ref_jv) <= 1e-12
    assert rel(jv32, ref_jv) <= 1e-5
    assert rel(diag, A.diagonal()) <= 1e-12
    assert nnz.value == A.nnz
    assert rel(csr, A.data) <= 1e-12


def _check_all(orc, u, du, outs, csr, nnz, A):
    r, r2, jv, jv32, diag = outs
    ref_r = orc.residual(u)
    assert rel(r, ref_r) <= 1e-12
    assert rel(r2, ref_r) <= 1e-12
    ref_jv = orc.jvp(u, du)
    assert rel(jv, ref_jv) <= 1e-12
    assert rel(jv32, ref_jv) <= 1e-5
    assert rel(diag, A.diagonal()) <= 1e-12
    assert nnz.value == A.nnz
    assert rel(csr, A.data) <= 1e-12


def test_user_boundary_qfunction_pressure(cuda, felib):
    """A user follower-pressure boundary q-function (AddBoundaryIntegral) on
    two sides, with a user Neo-Hookean domain integral, against the oracle's
    built-in pressure boundary integral (serac's boundary kernels)."""
    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=2)
    orc = O.OracleFunctional(m, 2, 3)
    orc.add_domain_integral(O.MAT_NEOHOOKEAN, PARAMS[O.MAT_NEOHOOKEAN])
    orc.add_boundary_integral(O.BMAT_PRESSURE, [3, 6], [0.7])
    u, du = fields(orc.ndofs, O.MAT_NEOHOOKEAN, seed=8)
    outs = [np.zeros(orc.ndofs) for _ in range(5)]
    A = orc.assemble(u)
    csr = np.zeros(A.nnz)
    nnz = ctypes.c_int64()
    V = np.ascontiguousarray(m.vertices)
    K, G = PARAMS[O.MAT_NEOHOOKEAN]
    mask = (1 << 2) | (1 << 5)
    rc = felib.frontend_neohookean_pressure(ctypes.c_double(K), ctypes.c_double(G), ctypes.c_double(0.7), mask, *dims,
                                            _p(V), _p(u), _p(du), *[_p(o) for o in outs], _p(csr), ctypes.byref(nnz))
    assert rc == 0
    _check_all(orc, u, du, outs, csr, nnz, A)


@pytest.mark.parametrize("p", [1, 2])
def test_user_boundary_qfunction_heat_flux(cuda, felib, p):
    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=3)
    orc = O.OracleFunctional(m, p, 1)
    orc.add_domain_integral(O.MAT_THERMAL_TEST, PARAMS[O.MAT_THERMAL_TEST])
    orc.add_boundary_integral(O.BMAT_HEAT_FLUX, [1, 4, 5], [0.3, 0.7, 1.1])
    u, du = fields(orc.ndofs, O.MAT_THERMAL_TEST, seed=9)
    outs = [np.zeros(orc.ndofs) for _ in range(5)]
    A = orc.assemble(u)
    csr = np.zeros(A.nnz)
    nnz = ctypes.c_int64()
    V = np.ascontiguousarray(m.vertices)
    mask = (1 << 0) | (1 << 3) | (1 << 4)
    rc = felib.frontend_thermal_flux(p, ctypes.c_double(0.3), ctypes.c_double(0.7), ctypes.c_double(1.1), mask, *dims,
                                     _p(V), _p(u), _p(du), *[_p(o) for o in outs], _p(csr), ctypes.byref(nnz))
    assert rc == 0
    _check_all(orc, u, du, outs, csr, nnz, A)


def test_shape_aware_user_qfunction_matches_oracle(cuda, felib):
    """sfx::ShapeAwareFunctional with a user Neo-Hookean q-function on a
    non-trilinear order-2 shape displacement."""
    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=2)
    mat = O.MAT_NEOHOOKEAN
    orc = O.OracleFunctional(m, 2, 3)
    orc.add_domain_integral(mat, PARAMS[mat])
    shape = np.random.default_rng(5).uniform(-0.02, 0.02, 3 * orc.nnodes)
    orc.set_shape(shape)
    u, du = fields(orc.ndofs, mat, seed=8)
    n = orc.ndofs
    outs = [np.zeros(n) for _ in range(5)]
    A = orc.assemble(u)
    csr = np.zeros(A.nnz)
    nnz = ctypes.c_int64()
    V = np.ascontiguousarray(m.vertices)
    K, G = PARAMS[mat]
    rc = felib.frontend_neohookean_shape(ctypes.c_double(K), ctypes.c_double(G), *dims, _p(V), _p(shape),
                                         ctypes.c_int64(shape.size), _p(u), _p(du), *[_p(o) for o in outs], _p(csr),
                                         ctypes.byref(nnz))
    assert rc == 0
    r, r2, jv, jv32, diag = outs
    assert rel(r, orc.residual(u)) <= 1e-12
    assert rel(r2, orc.residual(u)) <= 1e-12
    assert rel(jv, orc.jvp(u, du)) <= 1e-12
    assert rel(jv32, orc.jvp(u, du)) <= 1e-5
    assert rel(diag, A.diagonal()) <= 1e-12
    assert rel(csr, A.data) <= 1e-12


def test_user_qfunction_with_quadrature_state(cuda, felib):
    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=4)
    orc = O.OracleFunctional(m, 1, 3)
    prm = PARAMS[O.MAT_J2]
    orc.add_domain_integral(O.MAT_J2, prm)
    u, du = fields(orc.ndofs, O.MAT_J2, seed=13)
    n = orc.ndofs
    r_commit, r, jv = np.zeros(n), np.zeros(n), np.zeros(n)
    state = np.zeros((m.ne, 8, 10))
    V = np.ascontiguousarray(m.vertices)
    rc = felib.frontend_j2(*dims, _p(V), _p(u), _p(du), *[ctypes.c_double(x) for x in prm], _p(r_commit), _p(state),
                           _p(r), _p(jv))
    assert rc == 0
    assert rel(r_commit, orc.residual(u, update_state=True)) <= 1e-12
    assert np.abs(state - orc.state).max() <= 1e-12 * max(1.0, np.abs(orc.state).max())
    assert orc.state[..., 9].max() > 0
    assert rel(r, orc.residual(1.5 * u)) <= 1e-12
    assert rel(jv, orc.jvp(1.5 * u, du)) <= 1e-12


def _qoi_call(_fn):
    value, value2, action = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    return value, value2, action, [ctypes.byref(value), ctypes.byref(value2), ctypes.byref(action)]


@pytest.mark.parametrize("p", [1, 2])
def test_user_qoi_scalar(cuda, felib, p):
    """Functional<double(H1<p,1>)> with user domain and face integrands
    against the oracle's QOI_POLY_TEST (same mathematics, written separately)."""
    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=4)
    sides = [1, 3, 6]
    orc = O.OracleQoI(m, p, 1)
    orc.add_domain_integral(O.QOI_POLY_TEST)
    orc.add_boundary_integral(O.QOI_POLY_TEST, sides)
    rng = np.random.default_rng(40 + p)
    u = rng.standard_normal(orc.ndofs) * 0.1
    du = rng.standard_normal(orc.ndofs)
    grad = np.zeros(orc.ndofs)
    value, value2, action, refs = _qoi_call(None)
    mask = sum(1 << (s - 1) for s in sides)
    V = np.ascontiguousarray(m.vertices)
    rc = felib.frontend_qoi_poly(p, mask, *dims, _p(V), _p(u), _p(du), *refs, _p(grad))
    assert rc == 0
    ref_v, ref_g = orc.evaluate(u)
    assert abs(value.value - ref_v) <= 1e-12 * abs(ref_v)
    assert value2.value == value.value
    assert rel(grad, ref_g) <= 1e-12
    assert abs(action.value - ref_g @ du) <= 1e-12 * np.abs(ref_g).sum() * np.abs(du).max()


def test_user_qoi_vector_energy(cuda, felib):
    """A user stored-energy integrand plus u . n on faces (Q2 vector): the
    gradient matches the oracle (whose energy gradient is the pinned
    Neo-Hookean residual)."""
    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=6)
    K, G = PARAMS[O.MAT_NEOHOOKEAN]
    sides = [2, 6]
    orc = O.OracleQoI(m, 2, 3)
    orc.add_domain_integral(O.QOI_NEOHOOKEAN_ENERGY, [K, G])
    orc.add_boundary_integral(O.QOI_NORMAL_FIELD, sides)
    rng = np.random.default_rng(44)
    u = rng.standard_normal(orc.ndofs) * 0.01
    du = rng.standard_normal(orc.ndofs)
    grad = np.zeros(orc.ndofs)
    value, value2, action, refs = _qoi_call(None)
    mask = sum(1 << (s - 1) for s in sides)
    V = np.ascontiguousarray(m.vertices)
    rc = felib.frontend_qoi_energy(ctypes.c_double(K), ctypes.c_double(G), mask, *dims, _p(V), _p(u), _p(du), *refs,
                                   _p(grad))
    assert rc == 0
    ref_v, ref_g = orc.evaluate(u)
    # tr(F^T F) - 3 in the user integrand cancels: its value carries ~1e-16 / |H|^2 relative rounding
    assert abs(value.value - ref_v) <= 1e-10 * abs(ref_v)
    assert rel(grad, ref_g) <= 1e-12
    assert abs(action.value - ref_g @ du) <= 1e-12 * np.abs(ref_g).sum() * np.abs(du).max()


def test_user_transpose_action(cuda, felib):
    """Gradient::MultTranspose / MultTransposeF32 of a user Neo-Hookean +
    follower-pressure functional against the oracle's assembled transpose."""
    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=2)
    orc = O.OracleFunctional(m, 2, 3)
    orc.add_domain_integral(O.MAT_NEOHOOKEAN, PARAMS[O.MAT_NEOHOOKEAN])
    orc.add_boundary_integral(O.BMAT_PRESSURE, [3, 6], [0.7])
    u, v = fields(orc.ndofs, O.MAT_NEOHOOKEAN, seed=8)
    jt = np.zeros(orc.ndofs)
    jt32 = np.zeros(orc.ndofs)
    K, G = PARAMS[O.MAT_NEOHOOKEAN]
    mask = (1 << 2) | (1 << 5)
    V = np.ascontiguousarray(m.vertices)
    rc = felib.frontend_neohookean_pressure_transpose(ctypes.c_double(K), ctypes.c_double(G), ctypes.c_double(0.7),
                                                      mask, *dims, _p(V), _p(u), _p(v), _p(jt), _p(jt32))
    assert rc == 0
    ref = orc.jvp_transpose(u, v)
    assert rel(jt, ref) <= 1e-12
    assert rel(jt32, ref) <= 1e-5
    assert rel(ref, orc.jvp(u, v)) > 1e-6  # the follower pressure makes J non-symmetric


_i32p = ctypes.POINTER(ctypes.c_int32)


def _ip(a):
    return a.ctypes.data_as(_i32p)


def test_user_qfunctions_on_element_table(cuda, felib):
    """sfx::Mesh::FromTable (an imported element table: scrambled node ids,
    element order and element frames) with a user Neo-Hookean domain
    integral and a user follower pressure over a face list, against the
    oracle's table path."""
    from tests.problems import ScrambledTable

    m = mesh(3, 2, 2, perturb=0.1, seed=2)
    st = ScrambledTable(m, 2, seed=5)
    tm = O.TableHexMesh(2, st.table, st.corners, st.nn)
    fe, fs = st.faces_of_sides([3, 6])
    orc = O.OracleFunctional(tm, 2, 3)
    orc.add_domain_integral(O.MAT_NEOHOOKEAN, PARAMS[O.MAT_NEOHOOKEAN])
    orc.add_boundary_integral(O.BMAT_PRESSURE, (fe, fs), [0.7])
    u, du = fields(orc.ndofs, O.MAT_NEOHOOKEAN, seed=8)
    outs = [np.zeros(orc.ndofs) for _ in range(5)]
    A = orc.assemble(u)
    csr = np.zeros(A.nnz)
    nnz = ctypes.c_int64()
    table = np.ascontiguousarray(st.table, dtype=np.int32)
    corners = np.ascontiguousarray(st.corners)
    fe32, fs32 = np.ascontiguousarray(fe, dtype=np.int32), np.ascontiguousarray(fs, dtype=np.int32)
    fn = felib.frontend_table_neohookean_pressure
    fn.argtypes = ([ctypes.c_double] * 3 + [ctypes.c_int64] * 2 + [_i32p, _dp, ctypes.c_int64, _i32p, _i32p]
                   + [_dp] * 8 + [ctypes.POINTER(ctypes.c_int64)])
    K, G = PARAMS[O.MAT_NEOHOOKEAN]
    rc = fn(K, G, 0.7, m.ne, st.nn, _ip(table), _p(corners), len(fe32), _ip(fe32), _ip(fs32), _p(u), _p(du),
            *[_p(o) for o in outs], _p(csr), ctypes.byref(nnz))
    assert rc == 0
    _check_all(orc, u, du, outs, csr, nnz, A)


@pytest.mark.parametrize("p", [1, 2])
def test_user_qoi_on_element_table(cuda, felib, p):
    from tests.problems import ScrambledTable

    m = mesh(3, 2, 2, perturb=0.1, seed=4)
    st = ScrambledTable(m, p, seed=6)
    tm = O.TableHexMesh(p, st.table, st.corners, st.nn)
    fe, fs = st.faces_of_sides([1, 3, 6])
    orc = O.OracleQoI(tm, p, 1)
    orc.add_domain_integral(O.QOI_POLY_TEST)
    orc.add_boundary_integral(O.QOI_POLY_TEST, (fe, fs))
    rng = np.random.default_rng(50 + p)
    u = rng.standard_normal(orc.ndofs) * 0.1
    du = rng.standard_normal(orc.ndofs)
    grad = np.zeros(orc.ndofs)
    value, value2, action = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    table = np.ascontiguousarray(st.table, dtype=np.int32)
    corners = np.ascontiguousarray(st.corners)
    fe32, fs32 = np.ascontiguousarray(fe, dtype=np.int32), np.ascontiguousarray(fs, dtype=np.int32)
    fn = felib.frontend_table_qoi_poly
    fn.argtypes = ([ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _i32p, _dp, ctypes.c_int64, _i32p, _i32p, _dp, _dp]
                   + [ctypes.POINTER(ctypes.c_double)] * 3 + [_dp])
    rc = fn(p, m.ne, st.nn, _ip(table), _p(corners), len(fe32), _ip(fe32), _ip(fs32), _p(u), _p(du),
            ctypes.byref(value), ctypes.byref(value2), ctypes.byref(action), _p(grad))
    assert rc == 0
    ref_v, ref_g = orc.evaluate(u)
    assert abs(value.value - ref_v) <= 1e-12 * abs(ref_v)
    assert value2.value == value.value
    assert rel(grad, ref_g) <= 1e-12
    assert abs(action.value - ref_g @ du) <= 1e-12 * np.abs(ref_g).sum() * np.abs(du).max()


def test_user_shape_sensitivities(cuda, felib):
    """Front-end shape derivatives of user q-functions (ShapeJvp, ShapeVjp,
    and the QoI's ShapeGradient) against the C ABI's built-in Neo-Hookean,
    follower pressure, stored-energy and normal-displacement integrands on the
    same shape-displaced configuration."""
    import torch

    import serac_gb300 as sg

    dims = (3, 2, 2)
    m = mesh(*dims, perturb=0.1, seed=2)
    K, G = PARAMS[O.MAT_NEOHOOKEAN]
    sides = [3, 6]
    mask = sum(1 << (s - 1) for s in sides)
    nn = m.num_nodes(2)
    rng = np.random.default_rng(61)
    shape = rng.standard_normal(3 * nn) * 0.01
    u = rng.standard_normal(3 * nn) * 0.01
    dshape = rng.standard_normal(3 * nn)
    lam = rng.standard_normal(3 * nn)
    jvp, vjp, qsh = (np.zeros(3 * nn) for _ in range(3))
    V = np.ascontiguousarray(m.vertices)
    rc = felib.frontend_shape_sensitivity(ctypes.c_double(K), ctypes.c_double(G), ctypes.c_double(0.7), mask, *dims,
                                          _p(V), _p(shape), _p(u), _p(dshape), _p(lam), _p(jvp), _p(vjp), _p(qsh))
    assert rc == 0
    M = sg.Mesh.structured_hex(*dims, m.vertices)
    f = sg.Functional(M, sg.H1(2, 3))
    f.AddDomainIntegral(sg.NEOHOOKEAN, [K, G])
    f.AddBoundaryIntegral(sg.PRESSURE, sides, [0.7])
    f.set_shape_displacement(torch.tensor(shape, device=cuda))
    g = sg.ShapeGradient(f, 0.0, torch.tensor(u, device=cuda))
    assert rel(jvp, g(torch.tensor(dshape, device=cuda)).cpu().numpy()) <= 1e-10
    assert rel(vjp, g.MultTranspose(torch.tensor(lam, device=cuda)).cpu().numpy()) <= 1e-10
    q = sg.QoI(M, sg.H1(2, 3))
    q.AddDomainIntegral(sg.QOI_NEOHOOKEAN_ENERGY, [K, G])
    q.AddBoundaryIntegral(sg.QOI_NORMAL_FIELD, sides)
    q.set_shape_displacement(torch.tensor(shape, device=cuda))
    assert rel(qsh, q.shape_gradient(0.0, torch.tensor(u, device=cuda)).cpu().numpy()) <= 1e-9


@pytest.mark.parametrize("p", [1, 2])
def test_user_multi_field_qfunction(cuda, felib, p):
    """Functional<H1<p,3>(H1<p,3>, H1<p,3>, H1<p,1>, H1<p,1>)> with a user
    q-function (displacement, acceleration, two modulus-offset fields) under
    DependsOn<0, 1, 2, 3>: residual, derivative and transposed derivative
    with respect to every field against the oracle, 1e-12."""
    from tests.golden.make_golden import multi_fields

    dims = (3, 2, 2)
    V = O.box_vertices(*dims, 0.1, 9)
    rho, K0, G0 = 1.3, 5.0, 0.25
    orc = O.OracleMultiFunctional(O.StructuredHexMesh(*dims, V), p, [rho, K0, G0])
    N = orc.nnodes
    flds = multi_fields(N, 90 + p)
    rng = np.random.default_rng(p)
    felib.frontend_multi.restype = ctypes.c_int
    for w, c in enumerate(O.MULTI_COMPONENTS):
        d = rng.standard_normal(c * N)
        v = rng.standard_normal(3 * N)
        r, jv, jt = np.zeros(3 * N), np.zeros(3 * N), np.zeros(c * N)
        rc = felib.frontend_multi(p, *dims, _p(V), *[_p(f) for f in flds], w, _p(d), _p(v), ctypes.c_double(rho),
                                  ctypes.c_double(K0), ctypes.c_double(G0), _p(r), _p(jv), _p(jt))
        assert rc == 0
        assert rel(r, orc.residual(flds)) <= 1e-12
        assert rel(jv, orc.jvp(flds, w, d)) <= 1e-12, w
        assert rel(jt, orc.jvp_transpose(flds, w, v)) <= 1e-12, w
