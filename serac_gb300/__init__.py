"""serac_gb300 — GB300-native (sm_103a) weak-form engine with serac::Functional's
interface: residuals, Jacobian actions and CSR assembly of domain and boundary
integrals on hexahedral H1 meshes, computed by the sfx CUDA library."""
from .functional import (  # noqa: F401
    ELASTIC_TEST,
    HEAT,
    HEAT_FLUX,
    J2,
    NEOHOOKEAN,
    NONLINEAR_HEAT,
    PRESSURE,
    QOI_FIELD,
    QOI_MEASURE,
    QOI_NEOHOOKEAN_ENERGY,
    QOI_NORMAL_FIELD,
    QOI_POLY_TEST,
    QOI_POSITION,
    THERMAL_TEST,
    TRACTION,
    H1,
    Functional,
    Gradient,
    Mesh,
    QoI,
    QoIGradient,
    ShapeAwareFunctional,
    ShapeGradient,
    TableMesh,
    assemble,
    box_vertices,
    differentiate_wrt,
)
from .solver import CG, FGMRES, GMRES, JACOBI, JACOBI_CHEBYSHEV, LEARNED, NONE, NewtonSolver, SolverOptions  # noqa: F401,E402
