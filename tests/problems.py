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
