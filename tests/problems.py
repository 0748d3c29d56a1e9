"""Seeded test problems shared by the parity tests and the fixture generator."""
import numpy as np

from oracle import oracle as O

PARAMS = {
    O.MAT_HEAT: [1.3, 0.7],
    O.MAT_NEOHOOKEAN: [5.0, 0.25],
    O.MAT_J2: [100.0, 0.3, 1.0, 1.0],
    O.MAT_NONLINEAR_HEAT: [1.0, 0.5, 1.0],
    O.MAT_THERMAL_TEST: None,
    O.MAT_ELASTIC_TEST: None,
}
# displacement amplitude that keeps det F > 0 (Neo-Hookean) / reaches plasticity (J2)
AMPLITUDE = {O.MAT_NEOHOOKEAN: 0.02, O.MAT_J2: 0.02}


def mesh(nx, ny, nz, perturb=0.1, seed=1):
    return O.StructuredHexMesh(nx, ny, nz, O.box_vertices(nx, ny, nz, perturb, seed))


def fields(ndofs, mat, seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal(ndofs) * AMPLITUDE.get(mat, 0.3) * scale
    du = rng.standard_normal(ndofs)
    return u, du


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


# ---------------------------------------------------------------- element tables
_SIDE_OF = {(2, 0): 1, (1, 0): 2, (0, 1): 3, (1, 1): 4, (0, 0): 5, (2, 1): 6}
_DIR_OF = {v: k for k, v in _SIDE_OF.items()}


def cube_rotations():
    """The 24 proper rotations of the reference cube (signed permutation matrices, det +1)."""
    import itertools

    mats = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product([1, -1], repeat=3):
            R = np.zeros((3, 3), dtype=np.int64)
            for i in range(3):
                R[i, perm[i]] = signs[i]
            if round(np.linalg.det(R)) == 1:
                mats.append(R)
    return mats


def _local_map(R, n):
    """old lexicographic local index of every new local index under q' = R q
    (q = 2k - (n-1), centred index coordinates)."""
    p = n - 1
    out = np.empty(n ** 3, dtype=np.int64)
    for kz in range(n):
        for ky in range(n):
            for kx in range(n):
                qn = np.array([2 * kx - p, 2 * ky - p, 2 * kz - p])
                qo = R.T @ qn
                ko = (qo + p) // 2
                out[kx + n * (ky + n * kz)] = ko[0] + n * (ko[1] + n * ko[2])
    return out


class ScrambledTable:
    """An element table equivalent to a structured mesh: random node ids, a
    random element order and a random proper rotation of every element's
    local frame.  perm[old node] = new node; elem[k] = old element of new
    element k; rot[k] = rotation index."""

    def __init__(self, mesh, p, seed):
        rng = np.random.default_rng(seed)
        n = p + 1
        self.p, self.mesh = p, mesh
        self.nn = mesh.num_nodes(p)
        self.perm = rng.permutation(self.nn)
        self.elem = rng.permutation(mesh.ne)
        self.inv_elem = np.argsort(self.elem)
        rots = cube_rotations()
        self.R = [rots[i] for i in rng.integers(0, len(rots), mesh.ne)]
        conn = mesh.elem_nodes(p)
        Xe = mesh.elem_coords()  # (ne, 3, 8)
        self.table = np.empty((mesh.ne, n ** 3), dtype=np.int64)
        self.corners = np.empty((mesh.ne, 8, 3))
        for k in range(mesh.ne):
            e = self.elem[k]
            self.table[k] = self.perm[conn[e][_local_map(self.R[k], n)]]
            self.corners[k] = Xe[e].T[_local_map(self.R[k], 2)]

    def vdof_perm(self, c):
        """new vdof of every old vdof (byNODES)."""
        return (np.arange(c)[:, None] * self.nn + self.perm[None, :]).ravel()

    def to_new(self, x, c):
        out = np.empty_like(x)
        out[self.vdof_perm(c)] = x
        return out

    def faces_of_sides(self, sides):
        """(new element, new local side) of the faces on the given box sides."""
        elems, fsides = [], []
        m = self.mesh
        for s in sides:
            ax, hi = _DIR_OF[s]
            for e in range(m.ne):
                ex, ey, ez = e % m.nx, (e // m.nx) % m.ny, e // (m.nx * m.ny)
                idx = (ex, ey, ez)[ax]
                if idx != (((m.nx, m.ny, m.nz)[ax] - 1) if hi else 0):
                    continue
                k = self.inv_elem[e]
                d = np.zeros(3, dtype=np.int64)
                d[ax] = 1 if hi else -1
                dn = self.R[k] @ d
                axn = int(np.flatnonzero(dn)[0])
                elems.append(k)
                fsides.append(_SIDE_OF[(axn, 1 if dn[axn] > 0 else 0)])
        return np.array(elems, dtype=np.int32), np.array(fsides, dtype=np.int32)
