"""ORACLE — test infrastructure only.

CPU restatement of serac::Functional's global layer for structured hexahedral
H1 meshes on one rank (P = I): element restriction (gather / scatter-add),
domain + boundary integrals, Jacobian-vector products, element stiffness
assembly to CSR, Dirichlet elimination and plain FP64 Krylov / Newton
solvers.  The element arithmetic runs in ``liboracle.so`` (sfx_oracle.cpp).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's ``cpu_baseline`` leg
may import this module, and only as the checker / the timed CPU baseline.

Reference semantics followed:
  * Gather / ScatterAdd: E[(e*c + comp)*npe + j] = L[vdof]   (element_restriction.cpp:443-467)
  * byNODES vdof = comp * num_nodes + node                  (element_restriction.cpp:425-432)
  * residual: gather -> element kernel -> scatter            (functional.hpp:446-498)
  * Jv: same with the element Jacobian action               (functional.hpp:406-432)
  * CSR graph: sorted unique (row, col) pairs of every element's test x trial
    vdofs; values += K_e[trial][test]                        (dof_numbering.hpp:290-351, functional.hpp:590-644)
  * Dirichlet: residual rows set to zero (solid_mechanics.hpp:1118-1128);
    matrix rows and columns eliminated with a unit diagonal
    (boundary_condition_manager.hpp:91)
  * Krylov: textbook CG (Saad, Iterative Methods, Alg. 6.18) and restarted
    right-preconditioned GMRES (Alg. 9.5 in its flexible form) with Jacobi
  * Newton without line search (equation_solver.cpp:79-200, max_line_search_iterations = 0)
  * Quantities of interest (functional_qoi.inl:58-528, finite_element<g, QOI>):
    q det(J) w summed over points, dQ/du assembled from hand-derived partials
    (OracleQoI); checked against serac's own QOI element kernels when the
    reference library is built (OracleQoI.evaluate_reference)
  * Adjoint operators: J^T from the assembled matrix; shape sensitivities
    (dR/dp)^T lam and dQ/dp by central differences over the shape dofs
  * Imported element tables (TableHexMesh): element-node tables of one order
    with element corners, faces as (element, local side) pairs

Mesh numbering (shared with the product by specification, not by code):
  vertices   v(i,j,k) = i + (nx+1) (j + (ny+1) k), i in [0, nx]
  elements   e = ex + nx (ey + ny ez); local vertices lexicographic a + 2b + 4c
  H1 nodes   (p nx + 1)(p ny + 1)(p nz + 1) grid, node I + Nx (J + Ny K);
             element local node (kx, ky, kz) lexicographic -> (p ex + kx, p ey + ky, p ez + kz)
  boundary   sides 1..6 = z=0, y=0, x=1, y=1, x=0, z=1; each face is
             parametrised (s, t) so that dX/ds x dX/dt points outward; faces
             are ordered t-major within a side; local face node ks + (p+1) kt
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

MAT_HEAT, MAT_NEOHOOKEAN, MAT_J2, MAT_THERMAL_TEST, MAT_ELASTIC_TEST, MAT_NONLINEAR_HEAT = range(6)
BMAT_HEAT_FLUX, BMAT_TRACTION, BMAT_PRESSURE = range(3)
COMPONENTS = {MAT_HEAT: 1, MAT_NONLINEAR_HEAT: 1, MAT_THERMAL_TEST: 1, MAT_NEOHOOKEAN: 3, MAT_J2: 3, MAT_ELASTIC_TEST: 3}
NPARAMS = {MAT_HEAT: 2, MAT_NEOHOOKEAN: 2, MAT_J2: 4, MAT_NONLINEAR_HEAT: 3, MAT_THERMAL_TEST: 0, MAT_ELASTIC_TEST: 0}
BCOMPONENTS = {BMAT_HEAT_FLUX: 1, BMAT_TRACTION: 3, BMAT_PRESSURE: 3}
BNPARAMS = {BMAT_HEAT_FLUX: 3, BMAT_TRACTION: 6, BMAT_PRESSURE: 1}

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _declare(lib, prefix):
    f = getattr(lib, prefix + "geometric_factors")
    f.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
    f.restype = ctypes.c_int
    f = getattr(lib, prefix + "face_geometric_factors")
    f.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
    f.restype = ctypes.c_int
    f = getattr(lib, prefix + "domain")
    args = [ctypes.c_int] * 4 + [ctypes.c_double] + [_dp] * 5 + [_dp, ctypes.c_int, _dp]
    if prefix == "orc_":
        args = args + [ctypes.c_int]
    f.argtypes = args
    f.restype = ctypes.c_int
    f = getattr(lib, prefix + "boundary")
    f.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double] + [_dp] * 6
    f.restype = ctypes.c_int
    if prefix == "ref_" and hasattr(lib, "ref_qoi"):
        f = lib.ref_qoi
        f.argtypes = [ctypes.c_int] * 6 + [ctypes.c_double] + [_dp] * 5
        f.restype = ctypes.c_int


def lib():
    """The oracle's element-kernel library (built by ``make -C oracle``)."""
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])
        _LIB = ctypes.CDLL(path)
        _declare(_LIB, "orc_")
    return _LIB


def ref_lib():
    """serac's own element kernels compiled from the reference sources, or None
    where the reference tree is not present."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libserac_ref.so")
        if not os.path.exists(path):
            return None
        _REF = ctypes.CDLL(path)
        _declare(_REF, "ref_")
    return _REF


# --------------------------------------------------------------------- mesh
class StructuredHexMesh:
    """nx x ny x nz hexahedra with the given vertex coordinates ((nx+1)(ny+1)(nz+1), 3)."""

    def __init__(self, nx, ny, nz, vertices):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        assert self.vertices.shape[0] == (nx + 1) * (ny + 1) * (nz + 1)
        self.ne = nx * ny * nz

    def elem_vertex_ids(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        ex, ey, ez = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        ex, ey, ez = (a.transpose(2, 1, 0).ravel() for a in (ex, ey, ez))  # e = ex + nx(ey + ny ez)
        ids = np.empty((self.ne, 8), dtype=np.int64)
        for c in range(2):
            for b in range(2):
                for a in range(2):
                    ids[:, a + 2 * b + 4 * c] = (ex + a) + (nx + 1) * ((ey + b) + (ny + 1) * (ez + c))
        return ids

    def elem_coords(self):
        """(ne, 3, 8) vertex coordinates, lexicographic local order."""
        ids = self.elem_vertex_ids()
        return np.ascontiguousarray(self.vertices[ids].transpose(0, 2, 1))

    def num_nodes(self, p):
        return (p * self.nx + 1) * (p * self.ny + 1) * (p * self.nz + 1)

    def elem_nodes(self, p):
        nx, ny, nz = self.nx, self.ny, self.nz
        Nx, Ny = p * nx + 1, p * ny + 1
        e = np.arange(self.ne)
        ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
        n = p + 1
        conn = np.empty((self.ne, n ** 3), dtype=np.int64)
        for kz in range(n):
            for ky in range(n):
                for kx in range(n):
                    conn[:, kx + n * (ky + n * kz)] = (p * ex + kx) + Nx * ((p * ey + ky) + Ny * (p * ez + kz))
        return conn

    # side -> (fixed axis, fixed index(0/1), s axis, t axis)
    SIDES = {1: (2, 0, 1, 0), 2: (1, 0, 0, 2), 3: (0, 1, 1, 2), 4: (1, 1, 2, 0), 5: (0, 0, 2, 1), 6: (2, 1, 0, 1)}

    def boundary_faces(self, p, sides):
        """Face vertex coordinates (nf, 3, 4) and face node ids (nf, (p+1)^2)."""
        dims = (self.nx, self.ny, self.nz)
        Nn = (p * self.nx + 1, p * self.ny + 1, p * self.nz + 1)
        coords, nodes = [], []
        n = p + 1
        for side in sides:
            ax, hi, sa, ta = self.SIDES[side]
            fixed_v = dims[ax] if hi else 0
            for ft in range(dims[ta]):
                for fs in range(dims[sa]):
                    vids = []
                    for b in range(2):
                        for a in range(2):
                            idx = [0, 0, 0]
                            idx[ax] = fixed_v
                            idx[sa] = fs + a
                            idx[ta] = ft + b
                            vids.append(idx[0] + (self.nx + 1) * (idx[1] + (self.ny + 1) * idx[2]))
                    coords.append(self.vertices[vids].T)
                    fn = []
                    for kt in range(n):
                        for ks in range(n):
                            idx = [0, 0, 0]
                            idx[ax] = p * fixed_v
                            idx[sa] = p * fs + ks
                            idx[ta] = p * ft + kt
                            fn.append(idx[0] + Nn[0] * (idx[1] + Nn[1] * idx[2]))
                    nodes.append(fn)
        return np.ascontiguousarray(np.array(coords, dtype=np.float64)), np.array(nodes, dtype=np.int64)

    def boundary_nodes(self, p, sides):
        _, nodes = self.boundary_faces(p, sides)
        return np.unique(nodes.ravel())

    def node_coordinates(self, p):
        """(num_nodes, 3): the trilinear image of each element's Gauss-Lobatto
        nodes (nodes shared between elements get the same value)."""
        out = np.zeros((self.num_nodes(p), 3))
        conn = self.elem_nodes(p)
        Xe = self.elem_coords()  # (ne, 3, 8)
        g = np.linspace(0.0, 1.0, p + 1)
        n = p + 1
        for kz in range(n):
            for ky in range(n):
                for kx in range(n):
                    s = (g[kx], g[ky], g[kz])
                    w = np.array([(s[0] if a else 1 - s[0]) * (s[1] if b else 1 - s[1]) * (s[2] if c else 1 - s[2])
                                  for c in range(2) for b in range(2) for a in range(2)])
                    out[conn[:, kx + n * (ky + n * kz)]] = np.einsum("eiv,v->ei", Xe, w)
        return out


class TableHexMesh:
    """A conforming hexahedral mesh given by an element-node table of one
    order (lexicographic local node order, x fastest) and element corner
    coordinates (ne, 8, 3), as imported from an H1 element-dof table
    (element_restriction.cpp:216-277).  Faces are (element, local side)
    pairs with the sides parametrised in the element's own frame like the
    structured mesh's box sides."""

    SIDES = StructuredHexMesh.SIDES

    def __init__(self, order, elem_nodes, elem_vertices, num_nodes=None):
        self.order = order
        self.table = np.ascontiguousarray(elem_nodes, dtype=np.int64).reshape(-1, (order + 1) ** 3)
        self.corners = np.ascontiguousarray(elem_vertices, dtype=np.float64).reshape(-1, 8, 3)
        self.ne = self.table.shape[0]
        self.nn = int(self.table.max()) + 1 if num_nodes is None else int(num_nodes)

    def num_nodes(self, p):
        assert p == self.order
        return self.nn

    def elem_nodes(self, p):
        assert p == self.order
        return self.table

    def elem_coords(self):
        return np.ascontiguousarray(self.corners.transpose(0, 2, 1))

    def boundary_faces(self, p, faces):
        """faces: (elem array, side array) -> face vertex coordinates (nf, 3, 4), face nodes (nf, (p+1)^2)."""
        assert p == self.order
        elems, sides = (np.asarray(a, dtype=np.int64).ravel() for a in faces)
        n = p + 1
        coords, nodes = [], []
        for e, side in zip(elems, sides):
            ax, hi, sa, ta = self.SIDES[int(side)]
            cs = []
            for b in range(2):
                for a in range(2):
                    bb = [0, 0, 0]
                    bb[ax], bb[sa], bb[ta] = hi, a, b
                    cs.append(self.corners[e, bb[0] + 2 * bb[1] + 4 * bb[2]])
            coords.append(np.array(cs).T)
            fn = []
            for kt in range(n):
                for ks in range(n):
                    idx = [0, 0, 0]
                    idx[ax], idx[sa], idx[ta] = (p if hi else 0), ks, kt
                    fn.append(self.table[e, idx[0] + n * (idx[1] + n * idx[2])])
            nodes.append(fn)
        nf = len(nodes)
        return (np.ascontiguousarray(np.array(coords, dtype=np.float64).reshape(nf, 3, 4)),
                np.array(nodes, dtype=np.int64).reshape(nf, n * n))

    def boundary_nodes(self, p, faces):
        _, nodes = self.boundary_faces(p, faces)
        return np.unique(nodes.ravel())


def box_vertices(nx, ny, nz, perturb=0.0, seed=0):
    """Unit-cube vertex grid; interior vertices moved by U(-perturb*h, perturb*h)
    per coordinate with numpy's PCG64 generator seeded by ``seed``."""
    x = np.linspace(0.0, 1.0, nx + 1)
    y = np.linspace(0.0, 1.0, ny + 1)
    z = np.linspace(0.0, 1.0, nz + 1)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    if perturb > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-1.0, 1.0, size=V.shape) * perturb * np.array([1.0 / nx, 1.0 / ny, 1.0 / nz])
        i = np.arange(V.shape[0])
        ix, iy, iz = i % (nx + 1), (i // (nx + 1)) % (ny + 1), i // ((nx + 1) * (ny + 1))
        interior = (ix > 0) & (ix < nx) & (iy > 0) & (iy < ny) & (iz > 0) & (iz < nz)
        V[interior] += d[interior]
    return V


# ----------------------------------------------------------- element level
def basis_1d(p):
    """B[q, k], G[q, k]: the order-p Gauss-Lobatto Lagrange basis (nodes
    0, 1/p, ..., 1 for p <= 2) and its derivative at the p + 1 Gauss-Legendre
    points of [0, 1]."""
    nodes = np.linspace(0.0, 1.0, p + 1)
    t, _ = np.polynomial.legendre.leggauss(p + 1)
    x = 0.5 * (t + 1.0)
    B = np.ones((p + 1, p + 1))
    G = np.zeros((p + 1, p + 1))
    for k in range(p + 1):
        others = [j for j in range(p + 1) if j != k]
        for j in others:
            B[:, k] *= (x - nodes[j]) / (nodes[k] - nodes[j])
        for m in others:
            term = np.full(p + 1, 1.0 / (nodes[k] - nodes[m]))
            for j in others:
                if j != m:
                    term *= (x - nodes[j]) / (nodes[k] - nodes[j])
            G[:, k] += term
    return B, G


def geometric_factors(Xe, Q, use_ref=False):
    ne = Xe.shape[0]
    nq = Q ** 3
    Xq = np.zeros((ne, 3, nq))
    Jq = np.zeros((ne, 3, 3, nq))
    if use_ref:
        rc = ref_lib().ref_geometric_factors(Q, ne, _ptr(Xe), _ptr(Xq), _ptr(Jq))
    else:
        rc = lib().orc_geometric_factors(Q, ne, _ptr(Xe), _ptr(Xq), _ptr(Jq))
    assert rc == 0
    return Xq, Jq


def face_geometric_factors(Xf, Q, use_ref=False):
    nf = Xf.shape[0]
    nq = Q ** 2
    Xq = np.zeros((nf, 3, nq))
    Jq = np.zeros((nf, 2, 3, nq))
    if nf:
        if use_ref:
            rc = ref_lib().ref_face_geometric_factors(Q, nf, _ptr(Xf), _ptr(Xq), _ptr(Jq))
        else:
            rc = lib().orc_face_geometric_factors(Q, nf, _ptr(Xf), _ptr(Xq), _ptr(Jq))
        assert rc == 0
    return Xq, Jq


def element_kernel(mat, p, mode, uE, Xq, Jq, params=None, duE=None, state=None, update=False, t=0.0,
                   use_ref=False, nthreads=1):
    """mode 0 residual, 1 Jv, 2 K_e, on E-vectors (ne, c, npe)."""
    ne = uE.shape[0]
    c = COMPONENTS[mat]
    nd = (p + 1) ** 3 * c
    uE = np.ascontiguousarray(uE, dtype=np.float64)
    if duE is not None:
        duE = np.ascontiguousarray(duE, dtype=np.float64)
    out = np.zeros((ne, nd, nd) if mode == 2 else (ne, nd))
    prm = None
    if NPARAMS[mat]:
        prm = np.ascontiguousarray(np.broadcast_to(np.asarray(params, dtype=np.float64).reshape(-1, NPARAMS[mat]),
                                                   (ne, NPARAMS[mat])))
    if mat == MAT_J2 and state is None:
        state = np.zeros((ne, (p + 1) ** 3, 10))
    if ne == 0:
        return out
    if use_ref:
        rc = ref_lib().ref_domain(mat, p, mode, ne, t, _ptr(prm), _ptr(uE), _ptr(duE), _ptr(Xq), _ptr(Jq),
                                  _ptr(state), int(update), _ptr(out))
    else:
        rc = lib().orc_domain(mat, p, mode, ne, t, _ptr(prm), _ptr(uE), _ptr(duE), _ptr(Xq), _ptr(Jq),
                              _ptr(state), int(update), _ptr(out), nthreads)
    assert rc == 0, rc
    return out


def boundary_kernel(bmat, p, mode, uF, Xq, Jq, params, duF=None, t=0.0, use_ref=False):
    nf = uF.shape[0]
    c = BCOMPONENTS[bmat]
    nd = (p + 1) ** 2 * c
    out = np.zeros((nf, nd, nd) if mode == 2 else (nf, nd))
    if nf == 0:
        return out
    prm = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
    uF = np.ascontiguousarray(uF, dtype=np.float64)
    if duF is not None:
        duF = np.ascontiguousarray(duF, dtype=np.float64)
    fn = ref_lib().ref_boundary if use_ref else lib().orc_boundary
    rc = fn(bmat, p, mode, nf, t, _ptr(prm), _ptr(uF), _ptr(duF), _ptr(Xq), _ptr(Jq), _ptr(out))
    assert rc == 0, rc
    return out


# ------------------------------------------------------------ global layer
def gather(uL, conn, c, nnodes):
    """L-vector (byNODES) -> E-vector (ne, c, npe)."""
    u = uL.reshape(c, nnodes)
    return np.ascontiguousarray(u[:, conn].transpose(1, 0, 2)).reshape(conn.shape[0], c * conn.shape[1])


def scatter_add(E, conn, c, nnodes):
    out = np.zeros((c, nnodes))
    E = E.reshape(conn.shape[0], c, conn.shape[1])
    for k in range(c):
        np.add.at(out[k], conn.ravel(), E[:, k, :].ravel())
    return out.ravel()


def elem_vdofs(conn, c, nnodes):
    """(ne, c*npe) vdof ids, component-major per element."""
    return (np.arange(c)[None, :, None] * nnodes + conn[:, None, :]).reshape(conn.shape[0], -1)


class OracleFunctional:
    """Functional<H1<p,c>(H1<p,c>)> on a structured hex mesh (P = I)."""

    def __init__(self, mesh: StructuredHexMesh, p: int, c: int, use_ref: bool = False, nthreads: int = 1):
        self.mesh, self.p, self.c, self.use_ref, self.nthreads = mesh, p, c, use_ref, nthreads
        self.Q = p + 1
        self.nnodes = mesh.num_nodes(p)
        self.ndofs = self.nnodes * c
        self.conn = mesh.elem_nodes(p)
        self.Xq, self.Jq = geometric_factors(mesh.elem_coords(), self.Q, use_ref)
        self._geom0 = (self.Xq, self.Jq)
        self.shape = None
        self.domain = []
        self.boundary = []
        self._fgeom0 = []
        self.state = None

    def add_domain_integral(self, mat, params=None):
        assert COMPONENTS[mat] == self.c
        if mat == MAT_J2 and self.state is None:
            self.state = np.zeros((self.mesh.ne, self.Q ** 3, 10))
        self.domain.append((mat, params))

    def add_boundary_integral(self, bmat, sides, params):
        assert BCOMPONENTS[bmat] == self.c
        assert len(np.ravel(params)) == BNPARAMS[bmat], "wrong number of boundary parameters"
        Xf, fnodes = self.mesh.boundary_faces(self.p, sides)
        Xq, Jq = face_geometric_factors(Xf, self.Q, self.use_ref)
        self.boundary.append((bmat, params, fnodes, Xq, Jq))
        self._fgeom0.append((Xq, Jq))
        if self.shape is not None:
            self.set_shape(self.shape)

    def _apply(self, mode, u, du=None, update=False, t=0.0):
        c, N = self.c, self.nnodes
        out = np.zeros(self.ndofs)
        uE = gather(u, self.conn, c, N)
        duE = gather(du, self.conn, c, N) if du is not None else None
        for mat, params in self.domain:
            st = self.state if mat == MAT_J2 else None
            rE = element_kernel(mat, self.p, mode, uE, self.Xq, self.Jq, params, duE, st, update, t, self.use_ref,
                                self.nthreads)
            out += scatter_add(rE, self.conn, c, N)
        for bmat, params, fnodes, Xq, Jq in self.boundary:
            uF = gather(u, fnodes, c, N)
            duF = gather(du, fnodes, c, N) if du is not None else None
            rF = boundary_kernel(bmat, self.p, mode, uF, Xq, Jq, params, duF, t, self.use_ref)
            out += scatter_add(rF, fnodes, c, N)
        return out

    def set_shape(self, shape):
        """Shape displacement p (3 * nnodes, byNODES; None = none), as serac's
        ShapeAwareFunctional (shape_aware_functional.hpp:45-172): every integral
        is evaluated with position X + p and dx/dxi = dX/dxi + dp/dxi, which is
        the same as mapping the trial gradient by (I + dp/dX)^-1, scaling the
        outputs by det(I + dp/dX) (flux by (I + dp/dX)^-T) and the boundary
        weights by the area ratio."""
        self.shape = None if shape is None else np.array(shape, dtype=np.float64, copy=True)
        Xq0, Jq0 = self._geom0
        if self.shape is None:
            self.Xq, self.Jq = Xq0, Jq0
            for k, (Xf0, Jf0) in enumerate(self._fgeom0):
                bmat, params, fnodes, _, _ = self.boundary[k]
                self.boundary[k] = (bmat, params, fnodes, Xf0, Jf0)
            return
        B, G = basis_1d(self.p)
        n = self.p + 1
        P3 = self.shape.reshape(3, self.nnodes)
        # volume: phi[q, a], dphi[j][q, a] in lexicographic (x fastest) order
        Bz, By, Bx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        a_x, a_y, a_z = Bx.ravel(), By.ravel(), Bz.ravel()
        Qz, Qy, Qx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        q_x, q_y, q_z = Qx.ravel(), Qy.ravel(), Qz.ravel()
        bx, by, bz = B[q_x][:, a_x], B[q_y][:, a_y], B[q_z][:, a_z]
        gx, gy, gz = G[q_x][:, a_x], G[q_y][:, a_y], G[q_z][:, a_z]
        phi = bx * by * bz
        dphi = [gx * by * bz, bx * gy * bz, bx * by * gz]
        pE = P3[:, self.conn]  # (3, ne, npe)
        self.Xq = Xq0 + np.einsum("iea,qa->eiq", pE, phi)
        self.Jq = Jq0 + np.stack([np.einsum("iea,qa->eiq", pE, dphi[j]) for j in range(3)], axis=1)
        # faces: (s, t) lexicographic, s fastest
        Tt, Ts = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        a_s, a_t = Ts.ravel(), Tt.ravel()
        q_s, q_t = Ts.ravel(), Tt.ravel()
        fphi = B[q_s][:, a_s] * B[q_t][:, a_t]
        fds = G[q_s][:, a_s] * B[q_t][:, a_t]
        fdt = B[q_s][:, a_s] * G[q_t][:, a_t]
        for k, (Xf0, Jf0) in enumerate(self._fgeom0):
            bmat, params, fnodes, _, _ = self.boundary[k]
            pF = P3[:, fnodes]  # (3, nf, npf)
            Xf = Xf0 + np.einsum("ifa,qa->fiq", pF, fphi)
            Jf = Jf0 + np.stack([np.einsum("ifa,qa->fiq", pF, fds), np.einsum("ifa,qa->fiq", pF, fdt)], axis=1)
            self.boundary[k] = (bmat, params, fnodes, Xf, Jf)

    def residual(self, u, t=0.0, update_state=False):
        return self._apply(0, u, update=update_state, t=t)

    def jvp(self, u, du, t=0.0):
        return self._apply(1, u, du, t=t)

    def shape_vjp_fd(self, u, lam, base_shape=None, h=1e-6, t=0.0):
        """(dR/dp)^T lam by central differences over every shape dof (small
        meshes only); the shape is restored afterwards."""
        saved = self.shape
        p0 = np.zeros(3 * self.nnodes) if base_shape is None else np.asarray(base_shape, dtype=np.float64)
        out = np.zeros(3 * self.nnodes)
        for k in range(out.size):
            d = np.zeros_like(p0)
            d[k] = h
            self.set_shape(p0 + d)
            rp = self.residual(u, t)
            self.set_shape(p0 - d)
            rm = self.residual(u, t)
            out[k] = lam @ (rp - rm) / (2 * h)
        self.set_shape(saved)
        return out

    def jvp_transpose(self, u, v, t=0.0):
        """dR/du(u)^T v from the assembled matrix (pinned through assemble)."""
        return self.assemble(u, t).T @ v

    def csr_graph(self):
        vd = elem_vdofs(self.conn, self.c, self.nnodes)
        rows = np.repeat(vd, vd.shape[1], axis=1).ravel()
        cols = np.tile(vd, (1, vd.shape[1])).ravel()
        key = np.unique(rows * self.ndofs + cols)
        r, cl = key // self.ndofs, key % self.ndofs
        row_ptr = np.zeros(self.ndofs + 1, dtype=np.int64)
        np.add.at(row_ptr, r + 1, 1)
        return np.cumsum(row_ptr), cl.astype(np.int64)

    def assemble(self, u, t=0.0):
        """CSR (row_ptr, col, val) of dR/du; the graph holds every element's
        test x trial vdof pair (boundary faces add into it)."""
        import scipy.sparse as sp

        row_ptr, col = self.csr_graph()
        n = self.ndofs
        rows_of = np.repeat(np.arange(n, dtype=np.int64), np.diff(row_ptr))
        graph_keys = rows_of * n + col
        vals = np.zeros(col.shape[0])

        def add(K, vd):
            # K[e][trial j][test i] adds to row vd[e, i], column vd[e, j]
            nd = vd.shape[1]
            rows = np.tile(vd, (1, nd)).ravel()
            cols = np.repeat(vd, nd, axis=1).ravel()
            pos = np.searchsorted(graph_keys, rows * n + cols)
            np.add.at(vals, pos, K.ravel())

        uE = gather(u, self.conn, self.c, self.nnodes)
        vd = elem_vdofs(self.conn, self.c, self.nnodes)
        for mat, params in self.domain:
            st = self.state if mat == MAT_J2 else None
            K = element_kernel(mat, self.p, 2, uE, self.Xq, self.Jq, params, None, st, False, t, self.use_ref,
                               self.nthreads)
            add(K, vd)
        for bmat, params, fnodes, Xq, Jq in self.boundary:
            uF = gather(u, fnodes, self.c, self.nnodes)
            K = boundary_kernel(bmat, self.p, 2, uF, Xq, Jq, params, None, t, self.use_ref)
            add(K, elem_vdofs(fnodes, self.c, self.nnodes))
        # the graph holds every element pair, explicit zeros included
        return sp.csr_matrix((vals, col, row_ptr), shape=(n, n))


    def assemble_rows(self, u, rows, t=0.0, chunk=2048):
        """The CSR rows ``rows`` (sorted vdof ids) of dR/du from the domain
        integrals, for meshes whose full matrix is too large to assemble here:
        returns (row_ptr, col, val) of the sub-matrix A[rows, :], its graph the
        sorted unique columns that the elements containing each row's node
        pair it with, values summed in element order."""
        rows = np.asarray(rows, dtype=np.int64)
        n, c, N = self.ndofs, self.c, self.nnodes
        in_rows = np.zeros(n, dtype=bool)
        in_rows[rows] = True
        vd = elem_vdofs(self.conn, c, N)
        touching = np.nonzero(in_rows[vd].any(axis=1))[0]
        keys, vals = [], []
        uE = gather(u, self.conn, c, N)
        nd = vd.shape[1]
        for mat, params in self.domain:
            prm = None if not NPARAMS[mat] else np.asarray(params, dtype=np.float64).reshape(-1, NPARAMS[mat])
            per_element = prm is not None and prm.shape[0] == self.conn.shape[0] and prm.shape[0] > 1
            for k0 in range(0, touching.size, chunk):
                els = touching[k0:k0 + chunk]
                st = None if self.state is None or mat != MAT_J2 else np.ascontiguousarray(self.state[els])
                K = element_kernel(mat, self.p, 2, np.ascontiguousarray(uE[els]), np.ascontiguousarray(self.Xq[els]),
                                   np.ascontiguousarray(self.Jq[els]), prm[els] if per_element else prm, None, st,
                                   False, t, False, self.nthreads)
                # K[e][trial j][test i] adds to row vd[e, i], column vd[e, j]
                v = vd[els]
                r_ = np.broadcast_to(v[:, None, :], (els.size, nd, nd))
                c_ = np.broadcast_to(v[:, :, None], (els.size, nd, nd))
                sel = in_rows[r_]
                keys.append(r_[sel] * n + c_[sel])
                vals.append(K[sel])
        key = np.concatenate(keys)
        val = np.concatenate(vals)
        order = np.argsort(key, kind="stable")  # element order kept within a (row, col) pair
        key, val = key[order], val[order]
        first = np.ones(key.size, dtype=bool)
        first[1:] = key[1:] != key[:-1]
        starts = np.nonzero(first)[0]
        ukey = key[starts]
        uval = np.add.reduceat(val, starts)
        r_of, c_of = ukey // n, ukey % n
        pos = np.searchsorted(rows, r_of)
        row_ptr = np.zeros(rows.size + 1, dtype=np.int64)
        np.add.at(row_ptr, pos + 1, 1)
        return np.cumsum(row_ptr), c_of, uval


MAT_PARAM_NEOHOOKEAN = 16
MULTI_COMPONENTS = (3, 3, 1, 1)  # displacement, acceleration, bulk and shear modulus offsets


class OracleMultiFunctional:
    """Functional<test(displacement, acceleration, dK, dG)> on a structured hex
    mesh with the parameterized Neo-Hookean integrand of SolidMechanics
    (parameterized_solid_material.hpp:68-110 in solid_mechanics.hpp:809-850):
    every field byNODES on the order-p node grid, per-element parameters
    {density, K0, G0}.  residual(fields), jvp(fields, wrt, d),
    jvp_transpose(fields, wrt, v); ``use_ref`` evaluates residual and Jv with
    serac's own kernels (oracle/_ref)."""

    def __init__(self, mesh: StructuredHexMesh, p: int, params, nthreads: int = 1):
        self.mesh, self.p, self.nthreads = mesh, p, nthreads
        self.Q = p + 1
        self.nnodes = mesh.num_nodes(p)
        self.conn = mesh.elem_nodes(p)
        self.Xq, self.Jq = geometric_factors(mesh.elem_coords(), self.Q)
        ne = self.conn.shape[0]
        self.params = np.ascontiguousarray(np.broadcast_to(np.asarray(params, dtype=np.float64).reshape(-1, 3), (ne, 3)))
        L = lib()
        dp = _dp
        L.orc_domain_multi.argtypes = [ctypes.c_int] * 5 + [ctypes.c_double] + [dp] * 8 + [dp, ctypes.c_int]
        L.orc_domain_multi.restype = ctypes.c_int
        R = ref_lib()
        if R is not None:
            R.ref_domain_multi.argtypes = [ctypes.c_int] * 5 + [ctypes.c_double] + [dp] * 8 + [dp]
            R.ref_domain_multi.restype = ctypes.c_int

    def _gather(self, fields):
        return [np.ascontiguousarray(gather(np.asarray(f, dtype=np.float64), self.conn, c, self.nnodes))
                for f, c in zip(fields, MULTI_COMPONENTS)]

    def _call(self, mode, wrt, fields, dE, out_shape, use_ref=False, t=0.0):
        E = self._gather(fields)
        out = np.zeros(out_shape)
        ne = self.conn.shape[0]
        d = None if dE is None else np.ascontiguousarray(dE)
        if use_ref:
            rc = ref_lib().ref_domain_multi(MAT_PARAM_NEOHOOKEAN, self.p, mode, wrt, ne, t, _ptr(self.params), *map(_ptr, E),
                                            _ptr(d), _ptr(self.Xq), _ptr(self.Jq), _ptr(out))
        else:
            rc = lib().orc_domain_multi(MAT_PARAM_NEOHOOKEAN, self.p, mode, wrt, ne, t, _ptr(self.params), *map(_ptr, E),
                                        _ptr(d), _ptr(self.Xq), _ptr(self.Jq), _ptr(out), self.nthreads)
        assert rc == 0, rc
        return out

    def element_residuals(self, fields, use_ref=False):
        ne, nd = self.conn.shape
        return self._call(0, 0, fields, None, (ne, 3 * nd), use_ref)

    def residual(self, fields, use_ref=False):
        return scatter_add(self.element_residuals(fields, use_ref), self.conn, 3, self.nnodes)

    def jvp(self, fields, wrt, d, use_ref=False):
        c = MULTI_COMPONENTS[wrt]
        dE = gather(np.asarray(d, dtype=np.float64), self.conn, c, self.nnodes)
        ne, nd = self.conn.shape
        return scatter_add(self._call(1, wrt, fields, dE, (ne, 3 * nd), use_ref), self.conn, 3, self.nnodes)

    def element_matrices(self, fields, wrt, use_ref=False):
        """K_e with respect to argument wrt: [e][trial dof of wrt][test dof] (restatement); the
        reference's element_gradient_kernel layout for use_ref."""
        c = MULTI_COMPONENTS[wrt]
        ne, nd = self.conn.shape
        return self._call(2, wrt, fields, None, (ne, c * nd, 3 * nd), use_ref)

    def jvp_transpose(self, fields, wrt, v):
        c = MULTI_COMPONENTS[wrt]
        vE = gather(np.asarray(v, dtype=np.float64), self.conn, 3, self.nnodes)
        ne, nd = self.conn.shape
        return scatter_add(self._call(3, wrt, fields, vE, (ne, c * nd)), self.conn, c, self.nnodes)


QOI_MEASURE, QOI_POSITION, QOI_FIELD, QOI_NEOHOOKEAN_ENERGY, QOI_NORMAL_FIELD, QOI_POLY_TEST = range(6)


def _qoi_domain_point(kind, params, X, u, g, c):
    """q and its hand-derived partials at domain points: X (P, 3), u (P, c),
    g (P, c, 3) physical gradients -> q (P,), dq/du (P, c), dq/dg (P, c, 3).
    Integrands as in the product's C ABI (functional_qoi.inl semantics: the
    value is weighted by det(J) w)."""
    P = X.shape[0]
    q = np.zeros(P)
    du = np.zeros((P, c))
    dg = np.zeros((P, c, 3))
    if kind == QOI_MEASURE:
        q[:] = 1.0
    elif kind == QOI_POSITION:
        q = X @ np.asarray(params, dtype=np.float64)
    elif kind == QOI_FIELD:
        w = np.asarray(params, dtype=np.float64)
        q = u @ w
        du[:] = w
    elif kind == QOI_NEOHOOKEAN_ENERGY:
        # W = G/2 (|H|^2 + 2 tr H) - G ln J + lambda/2 (ln J)^2, dW/dH = G (F - F^-T) + lambda ln J F^-T
        K, G = params
        lam = K - 2.0 * G / 3.0
        F = g + np.eye(3)
        lnJ = np.log(np.linalg.det(F))
        q = 0.5 * G * (np.einsum("pij,pij->p", g, g) + 2.0 * np.einsum("pii->p", g)) - G * lnJ + 0.5 * lam * lnJ ** 2
        FinvT = np.linalg.inv(F).transpose(0, 2, 1)
        dg = G * (F - FinvT) + (lam * lnJ)[:, None, None] * FinvT
    elif kind == QOI_POLY_TEST:
        # X0^2 + sin X1 + X0 s^3 + (1 + X2)/2 |g|^2, s = sum_c u_c
        sm = u.sum(axis=1)
        q = X[:, 0] ** 2 + np.sin(X[:, 1]) + X[:, 0] * sm ** 3 + 0.5 * (1.0 + X[:, 2]) * np.einsum("pcj,pcj->p", g, g)
        du[:] = (3.0 * X[:, 0] * sm ** 2)[:, None]
        dg = (1.0 + X[:, 2])[:, None, None] * g
    else:
        raise ValueError(f"QoI kind {kind} not available on the domain")
    return q, du, dg


def _qoi_face_point(kind, params, X, J, u, gs, c):
    """q and partials at face points: X (P, 3), J (P, 3, 2) = dX/d(s, t),
    u (P, c), gs (P, c) = du/ds -> q (P,), dq/du (P, c), dq/d(du/ds) (P, c)."""
    P = X.shape[0]
    q = np.zeros(P)
    du = np.zeros((P, c))
    dgs = np.zeros((P, c))
    if kind == QOI_MEASURE:
        q[:] = 1.0
    elif kind == QOI_POSITION:
        q = X @ np.asarray(params, dtype=np.float64)
    elif kind == QOI_FIELD:
        w = np.asarray(params, dtype=np.float64)
        q = u @ w
        du[:] = w
    elif kind == QOI_NORMAL_FIELD:
        n = np.cross(J[:, :, 0], J[:, :, 1])
        n /= np.linalg.norm(n, axis=1)[:, None]
        q = np.einsum("pi,pi->p", n, u)
        du = n
    elif kind == QOI_POLY_TEST:
        # X0 - X1 + cos(s X1) + |du/ds|^2 / 4
        sm = u.sum(axis=1)
        q = X[:, 0] - X[:, 1] + np.cos(sm * X[:, 1]) + 0.25 * np.einsum("pc,pc->p", gs, gs)
        du[:] = (-np.sin(sm * X[:, 1]) * X[:, 1])[:, None]
        dgs = 0.5 * gs
    else:
        raise ValueError(f"QoI kind {kind} not available on faces")
    return q, du, dgs


def _tensor_basis(p):
    """Volume phi[q, a] and dphi[j][q, a]; face fphi[q, a], fds, fdt (lexicographic, x / s fastest)."""
    B, G = basis_1d(p)
    n = p + 1
    Kz, Ky, Kx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ax, ay, az = Kx.ravel(), Ky.ravel(), Kz.ravel()
    bx, by, bz = B[ax][:, ax], B[ay][:, ay], B[az][:, az]
    gx, gy, gz = G[ax][:, ax], G[ay][:, ay], G[az][:, az]
    phi = bx * by * bz
    dphi = [gx * by * bz, bx * gy * bz, bx * by * gz]
    Tt, Ts = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a_s, a_t = Ts.ravel(), Tt.ravel()
    fphi = B[a_s][:, a_s] * B[a_t][:, a_t]
    fds = G[a_s][:, a_s] * B[a_t][:, a_t]
    fdt = B[a_s][:, a_s] * G[a_t][:, a_t]
    return phi, dphi, fphi, fds, fdt


def _gl_weights(Q, dim):
    t, w = np.polynomial.legendre.leggauss(Q)
    w = 0.5 * w
    if dim == 3:
        return (w[None, None, :] * w[None, :, None] * w[:, None, None]).ravel()
    return (w[None, :] * w[:, None]).ravel()


class OracleQoI:
    """Functional<double(H1<p,c>)> (functional_qoi.inl:58-528) on a structured
    hex mesh: Q(u) = sum over elements and points of q det(J) w (+ faces with
    |dX/ds x dX/dt| w); dQ/du assembled from the integrands' hand-derived
    partials like a residual (Gradient::assemble, :422-475)."""

    def __init__(self, mesh: StructuredHexMesh, p: int, c: int, shape=None):
        self.mesh, self.p, self.c = mesh, p, c
        self.Q = p + 1
        self.nnodes = mesh.num_nodes(p)
        self.ndofs = self.nnodes * c
        self.conn = mesh.elem_nodes(p)
        self.Xq, self.Jq = geometric_factors(mesh.elem_coords(), self.Q)
        self.domain = []
        self.boundary = []
        self._bsides = []
        self._shape = None if shape is None else np.asarray(shape, dtype=np.float64)
        if self._shape is not None:
            self._apply_shape_domain()

    def _apply_shape_domain(self):
        phi, dphi, _, _, _ = _tensor_basis(self.p)
        P3 = self._shape.reshape(3, self.nnodes)[:, self.conn]
        self.Xq = self.Xq + np.einsum("iea,qa->eiq", P3, phi)
        self.Jq = self.Jq + np.stack([np.einsum("iea,qa->eiq", P3, dphi[j]) for j in range(3)], axis=1)

    def add_domain_integral(self, kind, params=None):
        self.domain.append((kind, params))

    def add_boundary_integral(self, kind, sides, params=None):
        Xf, fnodes = self.mesh.boundary_faces(self.p, sides)
        self._bsides.append(list(sides))
        Xq, Jq = face_geometric_factors(Xf, self.Q)
        if self._shape is not None:
            _, _, fphi, fds, fdt = _tensor_basis(self.p)
            P3 = self._shape.reshape(3, self.nnodes)[:, fnodes]
            Xq = Xq + np.einsum("ifa,qa->fiq", P3, fphi)
            Jq = Jq + np.stack([np.einsum("ifa,qa->fiq", P3, fds), np.einsum("ifa,qa->fiq", P3, fdt)], axis=1)
        self.boundary.append((kind, params, fnodes, Xq, Jq))

    def evaluate(self, u):
        """(Q(u), dQ/du)."""
        c, N, p = self.c, self.nnodes, self.p
        phi, dphi, fphi, fds, fdt = _tensor_basis(p)
        U = np.asarray(u, dtype=np.float64).reshape(c, N)
        value = 0.0
        grad = np.zeros((c, N))
        if self.domain:
            ne, nq = self.conn.shape[0], self.Q ** 3
            w = _gl_weights(self.Q, 3)
            J = self.Jq.transpose(0, 3, 2, 1)  # (e, q, i, j) = dX_i/dxi_j
            Jinv = np.linalg.inv(J)
            detJw = np.linalg.det(J) * w[None, :]
            X = self.Xq.transpose(0, 2, 1)  # (e, q, 3)
            uE = U[:, self.conn]  # (c, e, a)
            uq = np.einsum("cea,qa->eqc", uE, phi)
            gxi = np.stack([np.einsum("cea,qa->eqc", uE, dphi[j]) for j in range(3)], axis=-1)  # (e, q, c, j)
            gX = np.einsum("eqcj,eqji->eqci", gxi, Jinv)
            for kind, params in self.domain:
                q, dqu, dqg = _qoi_domain_point(kind, params, X.reshape(-1, 3), uq.reshape(-1, c),
                                                gX.reshape(-1, c, 3), c)
                value += float(np.sum(q.reshape(ne, nq) * detJw))
                src = dqu.reshape(ne, nq, c) * detJw[..., None]
                flx = np.einsum("eqci,eqji->eqcj", dqg.reshape(ne, nq, c, 3), Jinv) * detJw[..., None, None]
                gE = np.einsum("eqc,qa->cea", src, phi)
                for j in range(3):
                    gE += np.einsum("eqc,qa->cea", flx[..., j], dphi[j])
                for k in range(c):
                    np.add.at(grad[k], self.conn.ravel(), gE[k].ravel())
        for kind, params, fnodes, Xq, Jq in self.boundary:
            nf, nq = fnodes.shape[0], self.Q ** 2
            if nf == 0:
                continue
            w = _gl_weights(self.Q, 2)
            X = Xq.transpose(0, 2, 1).reshape(-1, 3)
            Jf = Jq.transpose(0, 3, 2, 1).reshape(-1, 3, 2)
            area = np.linalg.norm(np.cross(Jf[:, :, 0], Jf[:, :, 1]), axis=1).reshape(nf, nq) * w[None, :]
            uF = U[:, fnodes]
            uq = np.einsum("cfa,qa->fqc", uF, fphi).reshape(-1, c)
            gs = np.einsum("cfa,qa->fqc", uF, fds).reshape(-1, c)
            q, dqu, dqs = _qoi_face_point(kind, params, X, Jf, uq, gs, c)
            value += float(np.sum(q.reshape(nf, nq) * area))
            gF = np.einsum("fqc,qa->cfa", dqu.reshape(nf, nq, c) * area[..., None], fphi)
            gF += np.einsum("fqc,qa->cfa", dqs.reshape(nf, nq, c) * area[..., None], fds)
            for k in range(c):
                np.add.at(grad[k], fnodes.ravel(), gF[k].ravel())
        return value, grad.ravel()

    def evaluate_reference(self, u):
        """(Q(u), dQ/du) from serac's own QoI element kernels (evaluation_kernel_impl
        and element_gradient_kernel with the QOI test space, compiled into
        oracle/_ref), on the same geometric factors; None where the reference
        library is absent.  Integrands that depend on the field only."""
        R = ref_lib()
        if R is None or not hasattr(R, "ref_qoi"):
            return None
        c, N, p = self.c, self.nnodes, self.p
        value = 0.0
        grad = np.zeros(c * N)
        nd = c * (p + 1) ** 3
        uE = gather(u, self.conn, c, N)
        for kind, params in self.domain:
            prm = np.ascontiguousarray(np.asarray([0.0] if params is None else params, dtype=np.float64).ravel())
            ne = self.conn.shape[0]
            vals = np.zeros(ne)
            assert R.ref_qoi(kind, 0, p, c, 0, ne, 0.0, _ptr(prm), _ptr(uE), _ptr(self.Xq), _ptr(self.Jq),
                             _ptr(vals)) == 0
            ge = np.zeros((ne, nd))
            assert R.ref_qoi(kind, 0, p, c, 1, ne, 0.0, _ptr(prm), _ptr(uE), _ptr(self.Xq), _ptr(self.Jq),
                             _ptr(ge)) == 0
            value += float(vals.sum())
            grad += scatter_add(ge, self.conn, c, N)
        for kind, params, fnodes, Xq, Jq in self.boundary:
            prm = np.ascontiguousarray(np.asarray([0.0] if params is None else params, dtype=np.float64).ravel())
            nf = fnodes.shape[0]
            uF = gather(u, fnodes, c, N)
            vals = np.zeros(nf)
            Xq, Jq = np.ascontiguousarray(Xq), np.ascontiguousarray(Jq)
            assert R.ref_qoi(kind, 1, p, c, 0, nf, 0.0, _ptr(prm), _ptr(uF), _ptr(Xq), _ptr(Jq), _ptr(vals)) == 0
            gf = np.zeros((nf, c * (p + 1) ** 2))
            assert R.ref_qoi(kind, 1, p, c, 1, nf, 0.0, _ptr(prm), _ptr(uF), _ptr(Xq), _ptr(Jq), _ptr(gf)) == 0
            value += float(vals.sum())
            grad += scatter_add(gf, fnodes, c, N)
        return value, grad

    def value(self, u):
        return self.evaluate(u)[0]

    def shape_gradient_fd(self, u, base_shape=None, h=1e-6):
        """dQ/dp by central differences over every shape dof (small meshes only)."""
        p0 = np.zeros(3 * self.nnodes) if base_shape is None else np.asarray(base_shape, dtype=np.float64)
        out = np.zeros(3 * self.nnodes)

        def q_at(shape):
            other = OracleQoI(self.mesh, self.p, self.c, shape=shape)
            other.domain = list(self.domain)
            for (kind, params, _, _, _), sides in zip(self.boundary, self._bsides):
                other.add_boundary_integral(kind, sides, params)
            return other.value(u)

        for k in range(out.size):
            d = np.zeros_like(p0)
            d[k] = h
            out[k] = (q_at(p0 + d) - q_at(p0 - d)) / (2 * h)
        return out

    def gradient(self, u):
        return self.evaluate(u)[1]


class OracleLinearization:
    """The stored-derivative Jacobian of an OracleFunctional's domain
    integrals at u: the q-function derivative D is formed once per point
    (orc_linearize, evaluation_kernel_impl with differentiation) and each
    action is gather -> D . interpolate -> integrate -> node-owner scatter in
    C with OpenMP (orc_gather, orc_apply_linearization, orc_scatter:
    action_of_gradient_kernel, domain_integral_kernels.hpp:277-304).  Domain
    integrals only (no boundary integrals)."""

    def __init__(self, f, u, t=0.0, nthreads=None):
        assert not f.boundary, "domain integrals only"
        self.f = f
        self.threads = nthreads or f.nthreads
        L = lib()
        dp, i64p = _dp, ctypes.POINTER(ctypes.c_int64)
        L.orc_linearize.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] + [dp] * 5 + [dp, ctypes.c_int]
        L.orc_apply_linearization.argtypes = [ctypes.c_int] * 3 + [dp, dp, dp, ctypes.c_int]
        L.orc_gather.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int64, i64p, dp, dp,
                                 ctypes.c_int]
        L.orc_scatter.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, i64p, i64p, dp, dp, ctypes.c_int]
        self.L = L
        self.conn = np.ascontiguousarray(f.conn.astype(np.int64))
        ne, npe = self.conn.shape
        self.ne, self.npe = ne, npe
        order = np.argsort(self.conn.ravel(), kind="stable")
        self.node_ent = np.ascontiguousarray(order.astype(np.int64))
        node_ptr = np.zeros(f.nnodes + 1, dtype=np.int64)
        np.add.at(node_ptr, self.conn.ravel() + 1, 1)
        self.node_ptr = np.cumsum(node_ptr)
        c, nq = f.c, f.Q ** 3
        N = 4 * c
        uE = self.gather(np.ascontiguousarray(u, dtype=np.float64))
        self.D = []
        for mat, params in f.domain:
            prm = None
            if NPARAMS[mat]:
                prm = np.ascontiguousarray(np.broadcast_to(
                    np.asarray(params, dtype=np.float64).reshape(-1, NPARAMS[mat]), (ne, NPARAMS[mat])))
            st = f.state if mat == MAT_J2 else None
            D = np.zeros((ne, nq, N, N))
            rc = L.orc_linearize(mat, f.p, ne, t, _ptr(prm), _ptr(uE), _ptr(f.Xq), _ptr(f.Jq),
                                 _ptr(None if st is None else np.ascontiguousarray(st)), _ptr(D), self.threads)
            assert rc == 0, rc
            self.D.append(D)
        self._dE = np.zeros_like(uE)
        self._acc = np.zeros_like(uE)

    def gather(self, x):
        i64p = ctypes.POINTER(ctypes.c_int64)
        E = np.empty((self.ne, self.f.c * self.npe))
        self.L.orc_gather(self.ne, self.npe, self.f.c, self.f.nnodes, self.conn.ctypes.data_as(i64p), _ptr(x),
                          _ptr(E), self.threads)
        return E

    def scatter(self, E, out):
        i64p = ctypes.POINTER(ctypes.c_int64)
        self.L.orc_scatter(self.f.nnodes, self.npe, self.f.c, self.node_ptr.ctypes.data_as(i64p),
                           self.node_ent.ctypes.data_as(i64p), _ptr(E), _ptr(out), self.threads)
        return out

    def apply(self, x, out=None):
        """J(u) x."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty(self.f.ndofs) if out is None else out
        xE = self.gather(x)
        if len(self.D) == 1:
            self.L.orc_apply_linearization(self.f.p, self.f.c, self.ne, _ptr(self.D[0]), _ptr(xE),
                                           _ptr(self._dE), self.threads)
            return self.scatter(self._dE, out)
        self._acc[:] = 0.0
        for D in self.D:
            self.L.orc_apply_linearization(self.f.p, self.f.c, self.ne, _ptr(D), _ptr(xE), _ptr(self._dE),
                                           self.threads)
            self._acc += self._dE
        return self.scatter(self._acc, out)


def jacobian_diagonal(f, u, t=0.0, chunk=4096):
    """diag(dR/du) from the element matrices (domain integrals), in element chunks."""
    c, N = f.c, f.nnodes
    vd = elem_vdofs(f.conn, c, N)
    out = np.zeros(f.ndofs)
    uE = gather(u, f.conn, c, N)
    for mat, params in f.domain:
        prm = None if not NPARAMS[mat] else np.asarray(params, dtype=np.float64).reshape(-1, NPARAMS[mat])
        per_element = prm is not None and prm.shape[0] == f.conn.shape[0] and prm.shape[0] > 1
        for e0 in range(0, f.conn.shape[0], chunk):
            e1 = min(e0 + chunk, f.conn.shape[0])
            p_ch = prm[e0:e1] if per_element else prm
            st = None if f.state is None or mat != MAT_J2 else np.ascontiguousarray(f.state[e0:e1])
            K = element_kernel(mat, f.p, 2, uE[e0:e1], np.ascontiguousarray(f.Xq[e0:e1]),
                               np.ascontiguousarray(f.Jq[e0:e1]), p_ch, None, st, False, t, False, f.nthreads)
            np.add.at(out, vd[e0:e1].ravel(), np.einsum("eii->ei", K).ravel())
    return out


def newton_matrix_free(f, u0, ess, rel_tol=1e-10, abs_tol=0.0, lin_rtol=None, max_iter=30, t=0.0,
                       max_lin=50000):
    """Newton without line search (equation_solver.cpp:79-200) whose linear
    solves are Jacobi-preconditioned CG (Saad Alg. 6.18) on the
    Dirichlet-eliminated stored-derivative Jacobian, matrix-free
    (OracleLinearization): for meshes where a direct solve is out of reach.
    The converged solution does not depend on the linear solver, so by
    default each solve is only as tight as the step needs (inexact Newton,
    Eisenstat and Walker 1996): relative tolerance min(1e-2, 0.1 target / |r|),
    at least 1e-13; lin_rtol fixes it instead.  Returns (u, Newton
    iterations, final |r|, |r0|, total CG iterations)."""
    u = np.array(u0, dtype=np.float64, copy=True)
    mask = np.ones(f.ndofs)
    mask[ess] = 0.0
    r = f.residual(u, t=t)
    r[ess] = 0.0
    r0 = np.linalg.norm(r)
    it, lin_total = 0, 0
    for it in range(max_iter):
        if np.linalg.norm(r) <= max(rel_tol * r0, abs_tol):
            break
        lin = OracleLinearization(f, u, t)
        diag = jacobian_diagonal(f, u, t)
        diag[ess] = 1.0
        target = max(rel_tol * r0, abs_tol)
        eta = lin_rtol if lin_rtol is not None else max(1e-13, min(1e-2, 0.1 * target / np.linalg.norm(r)))
        du, k, _ = cg(lambda x: lin.apply(x * mask) * mask + x * (1.0 - mask), r, diag, rtol=eta,
                      maxiter=max_lin)
        lin_total += k
        u -= du
        r = f.residual(u, t=t)
        r[ess] = 0.0
    else:
        it = max_iter
    return u, it, np.linalg.norm(r), r0, lin_total


def newton_correction(f, u, ess, t=0.0, lin_rtol=1e-2, max_lin=50000):
    """One step of the oracle's own Newton iteration from u: the correction
    du = J(u)^-1 R(u) on the free rows (Dirichlet-eliminated, Jacobi-CG on
    the matrix-free stored-derivative Jacobian, to relative accuracy
    lin_rtol).  Near the solution Newton converges quadratically, so
    u - du is the oracle's converged solution up to O(|du|^2) + lin_rtol |du|:
    |du| measures how far u is from it.  Returns (du, |R(u)|, CG iterations)."""
    mask = np.ones(f.ndofs)
    mask[ess] = 0.0
    r = f.residual(u, t=t)
    r[ess] = 0.0
    lin = OracleLinearization(f, u, t)
    diag = jacobian_diagonal(f, u, t)
    diag[ess] = 1.0
    du, k, _ = cg(lambda x: lin.apply(x * mask) * mask + x * (1.0 - mask), r, diag, rtol=lin_rtol, maxiter=max_lin)
    return du, float(np.linalg.norm(r)), k


def warm_start_matrix_free(f, u, u_target, ess, t=0.0, lin_rtol=1e-3, max_lin=50000):
    """warm_start with the matrix-free Jacobi-CG linear solve (the predictor
    is only a starting point for Newton: its tolerance does not change the
    converged answer)."""
    mask = np.ones(f.ndofs)
    mask[ess] = 0.0
    d = np.zeros_like(u)
    d[ess] = u_target[ess] - u[ess]
    lin = OracleLinearization(f, u, t)
    rhs = -lin.apply(d)
    rhs[ess] = 0.0
    diag = jacobian_diagonal(f, u, t)
    diag[ess] = 1.0
    x, k, _ = cg(lambda y: lin.apply(y * mask) * mask + y * (1.0 - mask), rhs, diag, rtol=lin_rtol, maxiter=max_lin)
    x[ess] = 0.0
    return u + d + x, k


def eliminate_dirichlet(A, ess):
    """Zero the rows and columns of ``ess`` and put 1 on their diagonal."""
    import scipy.sparse as sp

    n = A.shape[0]
    keep = np.ones(n)
    keep[ess] = 0.0
    D = sp.diags(keep)
    A2 = (D @ A @ D).tocsr()
    A2 = A2 + sp.diags(1.0 - keep)
    A2 = A2.tocsr()
    A2.sort_indices()
    return A2


def _dot(a, b):
    """a . b without the BLAS library: its idle worker threads spin against
    the oracle's OpenMP threads and slow the matrix-free solves several-fold."""
    return float(np.einsum("i,i->", a, b))


def cg(apply_A, b, diag, rtol=1e-10, maxiter=10000):
    """Jacobi-preconditioned conjugate gradients; returns (x, iterations, ||r||/||b||)."""
    x = np.zeros_like(b)
    r = b.copy()
    z = r / diag
    p = z.copy()
    rz = _dot(r, z)
    nb = np.sqrt(_dot(b, b))
    if nb == 0:
        return x, 0, 0.0
    for it in range(1, maxiter + 1):
        Ap = apply_A(p)
        alpha = rz / _dot(p, Ap)
        x += alpha * p
        r -= alpha * Ap
        rn = np.sqrt(_dot(r, r)) / nb
        if rn < rtol:
            return x, it, rn
        np.divide(r, diag, out=z)
        rz_new = _dot(r, z)
        p *= rz_new / rz
        p += z
        rz = rz_new
    return x, maxiter, rn


def fgmres(apply_A, b, precond, rtol=1e-8, restart=50, maxiter=2000, atol=0.0):
    """Right-preconditioned flexible GMRES(restart) with modified Gram-Schmidt."""
    n = b.shape[0]
    x = np.zeros(n)
    nb = np.linalg.norm(b)
    if nb == 0:
        return x, 0, 0.0
    total = 0
    while total < maxiter:
        r = b - apply_A(x)
        beta = np.linalg.norm(r)
        if beta <= max(rtol * nb, atol):
            return x, total, beta / nb
        V = np.zeros((restart + 1, n))
        Zs = np.zeros((restart, n))
        H = np.zeros((restart + 1, restart))
        V[0] = r / beta
        g = np.zeros(restart + 1)
        g[0] = beta
        cs = np.zeros(restart)
        sn = np.zeros(restart)
        k = 0
        for k in range(restart):
            Zs[k] = precond(V[k])
            w = apply_A(Zs[k])
            for i in range(k + 1):
                H[i, k] = w @ V[i]
                w = w - H[i, k] * V[i]
            H[k + 1, k] = np.linalg.norm(w)
            if H[k + 1, k] > 0:
                V[k + 1] = w / H[k + 1, k]
            for i in range(k):
                t = cs[i] * H[i, k] + sn[i] * H[i + 1, k]
                H[i + 1, k] = -sn[i] * H[i, k] + cs[i] * H[i + 1, k]
                H[i, k] = t
            d = np.hypot(H[k, k], H[k + 1, k])
            cs[k], sn[k] = H[k, k] / d, H[k + 1, k] / d
            H[k, k] = d
            H[k + 1, k] = 0.0
            g[k + 1] = -sn[k] * g[k]
            g[k] = cs[k] * g[k]
            total += 1
            if abs(g[k + 1]) <= max(rtol * nb, atol) or total >= maxiter:
                break
        y = np.linalg.solve(np.triu(H[: k + 1, : k + 1]), g[: k + 1])
        x = x + y @ Zs[: k + 1]
    r = b - apply_A(x)
    return x, total, np.linalg.norm(r) / nb


def newton(f, u0, ess, rel_tol=1e-12, abs_tol=1e-14, max_iter=30, t=0.0):
    """Plain Newton with direct linear solves of the Dirichlet-eliminated
    Jacobian (equation_solver.cpp:79-200 without line search).  Returns
    (u, iterations, final ||r||)."""
    import scipy.sparse.linalg as spla

    u = np.array(u0, dtype=np.float64, copy=True)
    r = f.residual(u, t=t)
    r[ess] = 0.0
    r0 = np.linalg.norm(r)
    it = 0
    for it in range(max_iter):
        if np.linalg.norm(r) <= max(rel_tol * r0, abs_tol):
            break
        A = eliminate_dirichlet(f.assemble(u, t=t), ess)
        u -= spla.spsolve(A.tocsc(), r)
        r = f.residual(u, t=t)
        r[ess] = 0.0
    return u, it, np.linalg.norm(r)


def warm_start(f, u, u_target, ess, t=0.0):
    """Load-step predictor of SolidMechanics::warmStartDisplacement
    (solid_mechanics.hpp:1727-1770): d = essential-value increment, solve the
    Dirichlet-eliminated J(u) x = -J(u) d on the free rows, return u + d + x."""
    import scipy.sparse.linalg as spla

    d = np.zeros_like(u)
    d[ess] = u_target[ess] - u[ess]
    rhs = -f.jvp(u, d, t=t)
    rhs[ess] = 0.0
    x = spla.spsolve(eliminate_dirichlet(f.assemble(u, t=t), ess).tocsc(), rhs)
    x[ess] = 0.0
    return u + d + x
