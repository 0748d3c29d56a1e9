"""Generates the golden fixtures in this folder from serac's own element
kernels (oracle/_ref/libserac_ref.so, built by ``make -C oracle ref`` from the
reference sources) plus the oracle's global layer (gather / scatter / CSR).

Run from the repository root where the reference tree is present:
    make -C oracle ref && python tests/golden/make_golden.py [qoi|multi]
Inputs are regenerated from the seeds stored in each file; outputs are the
reference's numbers.  ``qoi`` writes only the quantity-of-interest fixtures
(values and gradients from serac's QOI element kernels); ``multi`` only the
multi-field fixtures (the parameterized Neo-Hookean integrand over
displacement, acceleration and two parameter fields, evaluated and
differentiated with respect to each argument by serac's own kernels).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.problems import PARAMS, fields, mesh  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

DOMAIN_CASES = [
    # name, material, order, dims, perturb, seed
    ("heat_p2", O.MAT_HEAT, 2, (2, 2, 2), 0.15, 1),
    ("heat_p1", O.MAT_HEAT, 1, (3, 2, 2), 0.15, 2),
    ("nonlinear_heat_p2", O.MAT_NONLINEAR_HEAT, 2, (2, 2, 1), 0.1, 3),
    ("thermal_test_p1", O.MAT_THERMAL_TEST, 1, (2, 2, 2), 0.1, 4),
    ("thermal_test_p2", O.MAT_THERMAL_TEST, 2, (2, 1, 1), 0.1, 5),
    ("neohookean_p2", O.MAT_NEOHOOKEAN, 2, (2, 2, 1), 0.1, 6),
    ("neohookean_p1", O.MAT_NEOHOOKEAN, 1, (2, 2, 2), 0.1, 7),
    ("elastic_test_p2", O.MAT_ELASTIC_TEST, 2, (2, 1, 1), 0.1, 8),
    ("j2_p1", O.MAT_J2, 1, (2, 2, 1), 0.1, 9),
    ("j2_p2", O.MAT_J2, 2, (1, 1, 1), 0.1, 10),
]

BOUNDARY_CASES = [
    # name, bmaterial, order, dims, sides, params, seed
    ("heat_flux_p2", O.BMAT_HEAT_FLUX, 2, (2, 2, 1), (1, 3, 6), [0.3, 0.7, 1.1], 11),
    ("traction_p1", O.BMAT_TRACTION, 1, (2, 1, 2), (2, 5, 6), [0.1, 0.2, 0.3, 0.5, -0.4, 0.2], 12),
    ("pressure_p2", O.BMAT_PRESSURE, 2, (1, 2, 1), (1, 2, 3, 4, 5, 6), [0.7], 13),
]


QOI_CASES = [
    # name, order, components, dims, domain integrands, face integrands, seed
    ("qoi_poly_p1", 1, 1, (2, 2, 2), [(O.QOI_POLY_TEST, None), (O.QOI_FIELD, [1.5])],
     [(O.QOI_POLY_TEST, [1, 3, 6], None)], 21),
    ("qoi_poly_p2", 2, 1, (2, 1, 2), [(O.QOI_POLY_TEST, None)], [(O.QOI_POLY_TEST, [2, 5], None),
                                                              (O.QOI_FIELD, [4], [0.5])], 22),
    ("qoi_energy_p2", 2, 3, (2, 1, 1), [(O.QOI_NEOHOOKEAN_ENERGY, [5.0, 0.25]), (O.QOI_FIELD, [1.0, 0.0, -2.0])],
     [(O.QOI_NORMAL_FIELD, [1, 6], None), (O.QOI_POLY_TEST, [3], None)], 23),
]


def qoi_case(name, p, c, dims, domain, faces, seed):
    m = mesh(*dims, perturb=0.15, seed=seed)
    q = O.OracleQoI(m, p, c)
    for kind, params in domain:
        q.add_domain_integral(kind, params)
    for kind, sides, params in faces:
        q.add_boundary_integral(kind, sides, params)
    rng = np.random.default_rng(seed)
    u = rng.standard_normal(q.ndofs) * (0.01 if c == 3 else 0.1)
    value, grad = q.evaluate_reference(u)
    out = {"dims": np.array(dims), "order": p, "components": c, "seed": seed, "u": u, "value": value,
           "gradient": grad}
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def domain_case(name, mat, p, dims, perturb, seed):
    m = mesh(*dims, perturb=perturb, seed=seed)
    f = O.OracleFunctional(m, p, O.COMPONENTS[mat], use_ref=True)
    f.add_domain_integral(mat, PARAMS[mat])
    u, du = fields(f.ndofs, mat, seed=seed)
    out = {"dims": np.array(dims), "order": p, "material": mat, "perturb": perturb, "seed": seed}
    if mat == O.MAT_J2:
        # commit the plastic state at u, then linearise at 1.5 u
        out["residual_commit"] = f.residual(u, update_state=True)
        out["state"] = f.state.copy()
        u = 1.5 * u
    out["residual"] = f.residual(u)
    out["jvp"] = f.jvp(u, du)
    A = f.assemble(u)
    out["csr_row_ptr"] = A.indptr.astype(np.int64)
    out["csr_col"] = A.indices.astype(np.int32)
    out["csr_val"] = A.data
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def boundary_case(name, bmat, p, dims, sides, params, seed):
    m = mesh(*dims, perturb=0.1, seed=seed)
    c = O.BCOMPONENTS[bmat]
    f = O.OracleFunctional(m, p, c, use_ref=True)
    f.add_boundary_integral(bmat, sides, params)
    rng = np.random.default_rng(seed)
    u = rng.standard_normal(f.ndofs) * 0.05
    du = rng.standard_normal(f.ndofs)
    out = {"dims": np.array(dims), "order": p, "bmaterial": bmat, "sides": np.array(sides), "params": np.array(params),
           "seed": seed, "u": u, "du": du}
    out["residual"] = f.residual(u)
    out["jvp"] = f.jvp(u, du)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


MULTI_CASES = [
    # name, order, dims, perturb, params {density, K0, G0}, seed
    ("param_neohookean_p2", 2, (2, 2, 1), 0.1, [1.3, 5.0, 0.25], 31),
    ("param_neohookean_p1", 1, (2, 2, 2), 0.1, [0.7, 3.0, 0.4], 32),
]


def multi_fields(nnodes, seed):
    """Seeded (displacement, acceleration, bulk and shear modulus offsets)."""
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(3 * nnodes) * 0.02, rng.standard_normal(3 * nnodes),
            0.5 * rng.standard_normal(nnodes), 0.05 * rng.standard_normal(nnodes)]


def multi_case(name, p, dims, perturb, params, seed):
    m = mesh(*dims, perturb=perturb, seed=seed)
    f = O.OracleMultiFunctional(m, p, params)
    flds = multi_fields(f.nnodes, seed)
    rng = np.random.default_rng(seed + 1000)
    out = {"dims": np.array(dims), "order": p, "perturb": perturb, "params": np.array(params), "seed": seed,
           "residual": f.residual(flds, use_ref=True)}
    for w, c in enumerate(O.MULTI_COMPONENTS):
        d = rng.standard_normal(c * f.nnodes)
        out[f"dir{w}"] = d
        out[f"jvp{w}"] = f.jvp(flds, w, d, use_ref=True)
        out[f"ke{w}"] = f.element_matrices(flds, w, use_ref=True)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


if __name__ == "__main__":
    if O.ref_lib() is None:
        sys.exit("reference checker not built: make -C oracle ref")
    if len(sys.argv) > 1 and sys.argv[1] == "multi":
        for case in MULTI_CASES:
            multi_case(*case)
        sys.exit(print("wrote", len(MULTI_CASES), "fixtures"))
    qoi_only = len(sys.argv) > 1 and sys.argv[1] == "qoi"
    if not qoi_only:
        for case in DOMAIN_CASES:
            domain_case(*case)
        for case in BOUNDARY_CASES:
            boundary_case(*case)
    for case in QOI_CASES:
        qoi_case(*case)
    if not qoi_only:
        for case in MULTI_CASES:
            multi_case(*case)
    print("wrote", len(QOI_CASES) + (0 if qoi_only else len(DOMAIN_CASES) + len(BOUNDARY_CASES) + len(MULTI_CASES)),
          "fixtures")
