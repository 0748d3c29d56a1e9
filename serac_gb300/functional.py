"""Python mirror of serac::Functional over the sfx C ABI.

    mesh = Mesh.structured_hex(nx, ny, nz, vertices)
    f = Functional(mesh, H1(order=2, components=3))       # Functional<H1<2,3>(H1<2,3>)>
    f.AddDomainIntegral(NEOHOOKEAN, params=[K, G])          # functional.hpp:286-317
    r = f(t, u)                                             # functional.hpp:502-513
    r, dRdu = f(t, differentiate_wrt(u))                    # functional.hpp:481-489
    dr = dRdu(du)                                           # Gradient::operator(), :562-566
    A = assemble(dRdu)                                      # functional.hpp:569-667 (CSR)

Vectors are torch CUDA tensors (float64; float32 for the FP32 Jacobian
action).  Like serac, the returned residual is a member buffer overwritten by
the next call (functional.hpp:740-741) unless ``out`` is given.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

HEAT, NEOHOOKEAN, J2, THERMAL_TEST, ELASTIC_TEST, NONLINEAR_HEAT = range(6)
HEAT_FLUX, TRACTION, PRESSURE = range(3)
COMPONENTS = {HEAT: 1, NONLINEAR_HEAT: 1, THERMAL_TEST: 1, NEOHOOKEAN: 3, J2: 3, ELASTIC_TEST: 3}
NPARAMS = {HEAT: 2, NEOHOOKEAN: 2, J2: 4, NONLINEAR_HEAT: 3, THERMAL_TEST: 0, ELASTIC_TEST: 0}
BNPARAMS = {HEAT_FLUX: 3, TRACTION: 6, PRESSURE: 1}
J2_STATE_DOUBLES = 10


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _require(t, dtype, n, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype or not t.is_contiguous() or t.numel() != n:
        raise ValueError(f"{name} must be a contiguous {dtype} tensor with {n} entries")


def _require_host(t, n, name):
    if not isinstance(t, torch.Tensor) or t.device.type != "cpu":
        raise TypeError(f"{name} must be a CPU tensor")
    if t.dtype != torch.float64 or not t.is_contiguous() or t.numel() != n:
        raise ValueError(f"{name} must be a contiguous float64 tensor with {n} entries")


@dataclass(frozen=True)
class H1:
    order: int
    components: int = 1


class Mesh:
    """Structured hexahedral mesh with trilinear geometry (buildCuboidMesh)."""

    def __init__(self, handle, nx, ny, nz, vertices):
        self._h = handle
        self.nx, self.ny, self.nz = nx, ny, nz
        self.vertices = vertices
        self.num_elements = nx * ny * nz

    @staticmethod
    def structured_hex(nx, ny, nz, vertices=None):
        if vertices is None:
            vertices = box_vertices(nx, ny, nz)
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        if v.shape[0] != (nx + 1) * (ny + 1) * (nz + 1):
            raise ValueError("vertex array has the wrong size")
        h = ctypes.c_void_p()
        _lib.call("sfx_mesh_create_structured_hex", nx, ny, nz, v.ctypes.data_as(_lib._dp), ctypes.byref(h))
        return Mesh(h, nx, ny, nz, v)

    def __del__(self):
        if getattr(self, "_h", None) and _lib._LIB is not None:
            _lib.load().sfx_mesh_destroy(self._h)
            self._h = None

    def node_coordinates(self, order):
        """(num_nodes, 3) positions of the H1 nodes of the given order: the
        trilinear image of each element's Gauss-Lobatto nodes."""
        p = order
        Nx, Ny, Nz = p * self.nx + 1, p * self.ny + 1, p * self.nz + 1
        idx = np.arange(Nx * Ny * Nz)
        I, J, K = idx % Nx, (idx // Nx) % Ny, idx // (Nx * Ny)
        gll = {1: np.array([0.0, 1.0]), 2: np.array([0.0, 0.5, 1.0])}[p]
        out = np.zeros((idx.size, 3))
        ijk = []
        for A, n in ((I, self.nx), (J, self.ny), (K, self.nz)):
            e = np.minimum(A // p, n - 1)
            ijk.append((e, gll[A - p * e]))
        (ex, sx), (ey, sy), (ez, sz) = ijk
        V = self.vertices.reshape(self.nz + 1, self.ny + 1, self.nx + 1, 3)
        for c in range(2):
            for b in range(2):
                for a in range(2):
                    w = (sx if a else 1 - sx) * (sy if b else 1 - sy) * (sz if c else 1 - sz)
                    out += w[:, None] * V[ez + c, ey + b, ex + a]
        return out

    def boundary_nodes(self, order, sides):
        """Sorted node ids on the given box sides (1: z=0, 2: y=0, 3: x=1,
        4: y=1, 5: x=0, 6: z=1)."""
        p = order
        Nx, Ny, Nz = p * self.nx + 1, p * self.ny + 1, p * self.nz + 1
        idx = np.arange(Nx * Ny * Nz)
        I, J, K = idx % Nx, (idx // Nx) % Ny, idx // (Nx * Ny)
        sel = np.zeros(idx.size, dtype=bool)
        tests = {1: K == 0, 2: J == 0, 3: I == Nx - 1, 4: J == Ny - 1, 5: I == 0, 6: K == Nz - 1}
        for s in sides:
            sel |= tests[s]
        return idx[sel]


class TableMesh:
    """A conforming hexahedral mesh as an element-node table of one order
    (an H1 element-dof table, lexicographic local order, the caller's node
    numbering) with element corner coordinates (num_elements, 8, 3); forms
    on it are built by sfx_form_create_from_table.  Boundaries are face
    lists (element, local side 1..6)."""

    def __init__(self, order, elem_nodes, elem_vertices, num_nodes=None):
        self.order = order
        self.table = np.ascontiguousarray(elem_nodes, dtype=np.int32).reshape(-1, (order + 1) ** 3)
        self.corners = np.ascontiguousarray(elem_vertices, dtype=np.float64).reshape(-1, 8, 3)
        self.num_elements = self.table.shape[0]
        self.num_nodes = int(self.table.max()) + 1 if num_nodes is None else int(num_nodes)

    def create(self, space, qoi=False):
        if space.order != self.order:
            raise ValueError("the space order must be the table's order")
        h = ctypes.c_void_p()
        _lib.call("sfx_qoi_create_from_table" if qoi else "sfx_form_create_from_table", self.order,
                  space.components, ctypes.c_int64(self.num_elements), ctypes.c_int64(self.num_nodes),
                  self.table.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), self.corners.ctypes.data_as(_lib._dp),
                  ctypes.byref(h))
        return h


def _face_arrays(faces):
    elems, sides = faces
    e = np.ascontiguousarray(np.asarray(elems, dtype=np.int32).ravel())
    s_ = np.ascontiguousarray(np.asarray(sides, dtype=np.int32).ravel())
    if e.size != s_.size:
        raise ValueError("face element and side arrays differ in length")
    return e, s_


def box_vertices(nx, ny, nz, perturb=0.0, seed=0):
    """Vertices of the unit cube grid; interior vertices moved uniformly by up
    to ``perturb`` times the cell size per coordinate (numpy PCG64, ``seed``)."""
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


class differentiate_wrt:
    """Marks the argument to linearise about (differentiate_wrt.hpp:12-42)."""

    def __init__(self, u):
        self.u = u


class Gradient:
    """dR/du at the linearisation point; an operator (functional.hpp:534-708)."""

    def __init__(self, form):
        self.form = form

    def mult(self, du, out=None, stream=None):
        """J du.  A CPU float64 du (and out) runs sfx_jvp_host: the copies to
        and from the device are made inside, overlapped with the kernels
        when the tensors are pinned."""
        f = self.form
        if isinstance(du, torch.Tensor) and du.device.type == "cpu":
            _require_host(du, f.ndofs, "du")
            out = torch.empty_like(du) if out is None else out
            _require_host(out, f.ndofs, "out")
            _lib.call("sfx_jvp_host", f._h, _dptr(du), _dptr(out), _stream(stream))
            return out
        if du.dtype == torch.float32:
            _require(du, torch.float32, f.ndofs, "du")
            out = torch.empty_like(du) if out is None else out
            _lib.call("sfx_jvp_f32", f._h, _dptr(du), _dptr(out), _stream(stream))
            return out
        _require(du, torch.float64, f.ndofs, "du")
        out = torch.empty_like(du) if out is None else out
        _lib.call("sfx_jvp", f._h, _dptr(du), _dptr(out), _stream(stream))
        return out

    Mult = mult

    def mult_transpose(self, v, out=None, stream=None):
        """dR/du^T v (mfem::Operator::MultTranspose): the adjoint action, from
        the stored tangent transposed (FP64, or FP32 for a float32 v)."""
        f = self.form
        if v.dtype == torch.float32:
            _require(v, torch.float32, f.ndofs, "v")
            out = torch.empty_like(v) if out is None else out
            _lib.call("sfx_jvp_transpose_f32", f._h, _dptr(v), _dptr(out), _stream(stream))
            return out
        _require(v, torch.float64, f.ndofs, "v")
        out = torch.empty_like(v) if out is None else out
        _lib.call("sfx_jvp_transpose", f._h, _dptr(v), _dptr(out), _stream(stream))
        return out

    MultTranspose = mult_transpose

    def element_action(self, du, out=None, stream=None):
        """Element-level action [e][component][node] before the scatter-add
        (FP64, or FP32 for a float32 du)."""
        f = self.form
        n = f.mesh.num_elements * f.space.components * (f.space.order + 1) ** 3
        if du.dtype == torch.float32:
            _require(du, torch.float32, f.ndofs, "du")
            out = torch.empty(n, dtype=torch.float32, device=du.device) if out is None else out
            _lib.call("sfx_jvp_element_f32", f._h, _dptr(du), _dptr(out), _stream(stream))
            return out
        _require(du, torch.float64, f.ndofs, "du")
        out = torch.empty(n, dtype=torch.float64, device=du.device) if out is None else out
        _lib.call("sfx_jvp_element", f._h, _dptr(du), _dptr(out), _stream(stream))
        return out

    def __call__(self, du):
        return self.mult(du)


class Functional:
    """Functional<H1<p,c>(H1<p,c>)> on a structured hex mesh."""

    def __init__(self, mesh, space: H1):
        self.mesh = mesh
        self.space = space
        if isinstance(mesh, TableMesh):
            h = mesh.create(space)
        else:
            h = ctypes.c_void_p()
            _lib.call("sfx_form_create", mesh._h, space.order, space.components, ctypes.byref(h))
        self._h = h
        n = ctypes.c_int64()
        _lib.call("sfx_form_num_dofs", h, ctypes.byref(n))
        self.ndofs = n.value
        self.num_nodes = self.ndofs // space.components
        self.gradient = Gradient(self)
        self._out = None
        self._materials = []

    def __del__(self):
        if getattr(self, "_h", None) and _lib._LIB is not None:
            _lib.load().sfx_form_destroy(self._h)
            self._h = None

    # --------------------------------------------------------------- setup
    def AddDomainIntegral(self, material, params=None, per_element=False):
        np_ = NPARAMS[material]
        p = None
        if np_:
            arr = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
            expect = self.mesh.num_elements * np_ if per_element else np_
            if arr.size != expect:
                raise ValueError(f"expected {expect} parameters, got {arr.size}")
            self._params_keepalive = arr
            p = arr.ctypes.data_as(_lib._dp)
        _lib.call("sfx_form_add_domain_integral", self._h, material, p, int(per_element))
        self._materials.append(material)

    add_domain_integral = AddDomainIntegral
    AddVolumeIntegral = AddDomainIntegral

    def set_parameters(self, params, per_element=False, integral=0):
        """Replace the material parameters of a domain integral (the order of
        AddDomainIntegral calls) in place; linearise again afterwards."""
        material = self._materials[integral]
        np_ = NPARAMS[material]
        arr = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
        expect = self.mesh.num_elements * np_ if per_element else np_
        if arr.size != expect:
            raise ValueError(f"expected {expect} parameters, got {arr.size}")
        _lib.call("sfx_set_param_field", self._h, int(integral), arr.ctypes.data_as(_lib._dp), int(per_element))

    def AddBoundaryIntegral(self, material, sides=None, params=None, faces=None):
        """Over the box sides (structured meshes) or a face list
        faces = (element array, local side array)."""
        arr = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
        if material in BNPARAMS and arr.size != BNPARAMS[material]:
            raise ValueError(f"boundary material {material} takes {BNPARAMS[material]} parameters, got {arr.size}")
        if faces is not None:
            e, s_ = _face_arrays(faces)
            _lib.call("sfx_form_add_boundary_integral_faces", self._h, material, ctypes.c_int64(e.size),
                      e.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), s_.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                      arr.ctypes.data_as(_lib._dp))
            return
        mask = 0
        for s in sides:
            mask |= 1 << (s - 1)
        _lib.call("sfx_form_add_boundary_integral", self._h, material, mask, arr.ctypes.data_as(_lib._dp))

    add_boundary_integral = AddBoundaryIntegral
    AddSurfaceIntegral = AddBoundaryIntegral

    STORED_TANGENT, RECOMPUTE = 0, 1

    def set_jvp_mode(self, mode):
        """STORED_TANGENT (default): the q-function derivative is stored at each
        quadrature point by linearize(); RECOMPUTE: every Jacobian action
        re-evaluates the q-function on dual numbers."""
        _lib.call("sfx_form_set_jvp_mode", self._h, int(mode))

    TANGENT_F32, TANGENT_F16 = 0, 1

    def set_tangent_storage(self, storage):
        """Storage of the tangent copy streamed by the FP32 action (the inner
        Krylov operator): TANGENT_F32 (default) or TANGENT_F16 (order 2)."""
        _lib.call("sfx_form_set_tangent_storage", self._h, int(storage))

    def set_shape_displacement(self, shape, stream=None):
        """Evaluate every integral on the configuration X + shape (float64 CUDA
        tensor, 3 * num_nodes, byNODES; None = the reference configuration),
        as serac's ShapeAwareFunctional.  Linearise again afterwards."""
        if shape is None:
            _lib.call("sfx_form_set_shape_displacement", self._h, None, _stream(stream))
        else:
            _require(shape, torch.float64, 3 * self.num_nodes, "shape")
            _lib.call("sfx_form_set_shape_displacement", self._h, _dptr(shape), _stream(stream))

    def updateQdata(self, flag: bool):
        _lib.call("sfx_update_qdata", self._h, int(bool(flag)))

    def qdata(self):
        n = ctypes.c_int64()
        _lib.call("sfx_qdata_size", self._h, ctypes.byref(n))
        out = np.zeros(n.value)
        if n.value:
            _lib.call("sfx_get_qdata", self._h, out.ctypes.data_as(_lib._dp))
        return out

    def set_qdata(self, host):
        a = np.ascontiguousarray(host, dtype=np.float64).ravel()
        _lib.call("sfx_set_qdata", self._h, a.ctypes.data_as(_lib._dp))

    # ----------------------------------------------------------- evaluation
    def residual(self, t, u, out=None, stream=None):
        _require(u, torch.float64, self.ndofs, "u")
        out = torch.empty_like(u) if out is None else out
        _lib.call("sfx_residual", self._h, float(t), _dptr(u), _dptr(out), _stream(stream))
        return out

    def linearize(self, t, u, out=None, stream=None):
        _require(u, torch.float64, self.ndofs, "u")
        _lib.call("sfx_linearize", self._h, float(t), _dptr(u), _dptr(out), _stream(stream))
        return self.gradient

    def __call__(self, t, arg, out=None):
        if isinstance(arg, differentiate_wrt):
            if self._out is None:
                self._out = torch.empty(self.ndofs, dtype=torch.float64, device=arg.u.device)
            r = self._out if out is None else out
            self.linearize(t, arg.u, r)
            return r, self.gradient
        if out is None:
            if self._out is None:
                self._out = torch.empty(self.ndofs, dtype=torch.float64, device=arg.device)
            out = self._out
        return self.residual(t, arg, out)

    # ------------------------------------------------------------ assembly
    def csr_graph(self, stream=None):
        n = ctypes.c_int64()
        _lib.call("sfx_csr_nnz", self._h, ctypes.byref(n))
        row_ptr = torch.empty(self.ndofs + 1, dtype=torch.int64, device="cuda")
        col = torch.empty(n.value, dtype=torch.int32, device="cuda")
        _lib.call("sfx_csr_graph", self._h, _dptr(row_ptr), _dptr(col), _stream(stream))
        return row_ptr, col

    def assemble_values(self, out=None, stream=None):
        n = ctypes.c_int64()
        _lib.call("sfx_csr_nnz", self._h, ctypes.byref(n))
        out = torch.empty(n.value, dtype=torch.float64, device="cuda") if out is None else out
        _lib.call("sfx_assemble_csr", self._h, _dptr(out), _stream(stream))
        return out

    def assemble_diagonal(self, out=None, stream=None):
        out = torch.empty(self.ndofs, dtype=torch.float64, device="cuda") if out is None else out
        _lib.call("sfx_assemble_diagonal", self._h, _dptr(out), _stream(stream))
        return out


class ShapeGradient:
    """dR/dp at (t, shape, u): the derivative of the shape-aware residual with
    respect to the shape displacement, as an operator on shape directions."""

    def __init__(self, functional, t, u):
        self.functional = functional
        self.t = t
        self.u = u.clone()

    def mult(self, dshape, out=None, stream=None):
        f = self.functional
        _require(dshape, torch.float64, 3 * f.num_nodes, "dshape")
        out = torch.empty(f.ndofs, dtype=torch.float64, device=dshape.device) if out is None else out
        _lib.call("sfx_shape_jvp", f._h, float(self.t), _dptr(self.u), _dptr(dshape), _dptr(out), _stream(stream))
        return out

    Mult = mult

    def mult_transpose(self, lam, out=None, stream=None):
        """(dR/dp)^T lam (3 * num_nodes): the adjoint shape sensitivity
        (computeTimestepShapeSensitivity, solid_mechanics.hpp:1421-1431)."""
        f = self.functional
        _require(lam, torch.float64, f.ndofs, "lam")
        out = torch.empty(3 * f.num_nodes, dtype=torch.float64, device=lam.device) if out is None else out
        _lib.call("sfx_shape_vjp", f._h, float(self.t), _dptr(self.u), _dptr(lam), _dptr(out), _stream(stream))
        return out

    MultTranspose = mult_transpose

    def __call__(self, dshape):
        return self.mult(dshape)


class ShapeAwareFunctional:
    """ShapeAwareFunctional<H1<p,3>, H1<p,c>(H1<p,c>)> (shape_aware_functional.hpp:330-560):
    the shape displacement is the first argument after time and is held
    fixed by the evaluation.

        saf = ShapeAwareFunctional(mesh, H1(2, 3), H1(2, 3))
        saf.AddDomainIntegral(NEOHOOKEAN, [K, G])
        r = saf(t, shape, u)
        r, dRdu = saf(t, shape, differentiate_wrt(u))
        r, dRdp = saf(t, differentiate_wrt(shape), u)     # dRdp(dshape)
    """

    def __init__(self, mesh: Mesh, shape_space: H1, space: H1):
        if shape_space.components != 3 or shape_space.order != space.order:
            raise ValueError("the shape space must be H1 with 3 components and the trial space's order")
        self.functional = Functional(mesh, space)
        self.ndofs = self.functional.ndofs
        self._shape_key = None

    def AddDomainIntegral(self, *a, **k):
        return self.functional.AddDomainIntegral(*a, **k)

    def AddBoundaryIntegral(self, *a, **k):
        return self.functional.AddBoundaryIntegral(*a, **k)

    def updateQdata(self, flag):
        return self.functional.updateQdata(flag)

    def _use(self, shape):
        key = (shape.data_ptr(), shape._version)
        if key != self._shape_key:
            self.functional.set_shape_displacement(shape)
            self._shape_key = key

    def __call__(self, t, shape, arg, out=None):
        if isinstance(shape, differentiate_wrt):
            self._use(shape.u)
            r = self.functional(t, arg, out)
            return r, ShapeGradient(self.functional, t, arg)
        self._use(shape)
        return self.functional(t, arg, out)


QOI_MEASURE, QOI_POSITION, QOI_FIELD, QOI_NEOHOOKEAN_ENERGY, QOI_NORMAL_FIELD, QOI_POLY_TEST = range(6)


def _qoi_nparams(kind, c, boundary):
    n = {QOI_MEASURE: 0, QOI_POSITION: 3, QOI_FIELD: c, QOI_POLY_TEST: 0}
    if not boundary and c == 3:
        n[QOI_NEOHOOKEAN_ENERGY] = 2
    if boundary and c == 3:
        n[QOI_NORMAL_FIELD] = 0
    if kind not in n:
        raise ValueError(f"QoI kind {kind} is not available {'on faces' if boundary else 'on the domain'} "
                         f"for {c} components")
    return n[kind]


class QoIGradient:
    """dQ/du at (t, u) of a quantity of interest (functional_qoi.inl:407-477):
    ``g(du)`` is the directional derivative (Gradient::operator(), :420) and
    ``assemble(g)`` the gradient vector (Gradient::assemble, :422-475)."""

    def __init__(self, qoi, t, u):
        self.qoi = qoi
        self.t = t
        self.u = u.clone()

    def action(self, du, out=None, stream=None):
        """dQ/du du as a one-element float64 CUDA tensor."""
        q = self.qoi
        _require(du, torch.float64, q.ndofs, "du")
        out = torch.empty(1, dtype=torch.float64, device=du.device) if out is None else out
        _lib.call("sfx_qoi_action", q._h, float(self.t), _dptr(self.u), _dptr(du), _dptr(out), _stream(stream))
        return out

    def __call__(self, du):
        return float(self.action(du).item())

    def assemble(self, out=None, stream=None):
        q = self.qoi
        out = torch.empty(q.ndofs, dtype=torch.float64, device=self.u.device) if out is None else out
        _lib.call("sfx_qoi_gradient", q._h, float(self.t), _dptr(self.u), None, _dptr(out), _stream(stream))
        return out


class QoI:
    """Functional<double(H1<p,c>)>: a quantity of interest (functional_qoi.inl:58-528).

        q = QoI(mesh, H1(2, 3))
        q.AddDomainIntegral(QOI_NEOHOOKEAN_ENERGY, [K, G])    # :159-189
        q.AddBoundaryIntegral(QOI_NORMAL_FIELD, sides=[6])    # :201-228
        value = q(t, u)                                       # :379-392
        value, dQdu = q(t, differentiate_wrt(u))
        dQdu(du); assemble(dQdu)                              # :420, :422-475
    """

    def __init__(self, mesh, space: H1):
        self.mesh = mesh
        self.space = space
        if isinstance(mesh, TableMesh):
            h = mesh.create(space, qoi=True)
        else:
            h = ctypes.c_void_p()
            _lib.call("sfx_qoi_create", mesh._h, space.order, space.components, ctypes.byref(h))
        self._h = h
        n = ctypes.c_int64()
        _lib.call("sfx_form_num_dofs", h, ctypes.byref(n))
        self.ndofs = n.value
        self.num_nodes = self.ndofs // space.components
        self._keep = []

    def __del__(self):
        if getattr(self, "_h", None) and _lib._LIB is not None:
            _lib.load().sfx_form_destroy(self._h)
            self._h = None

    def _params(self, kind, params, boundary):
        n = _qoi_nparams(kind, self.space.components, boundary)
        if n == 0:
            return None
        arr = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
        if arr.size != n:
            raise ValueError(f"QoI kind {kind} takes {n} parameters, got {arr.size}")
        self._keep.append(arr)
        return arr.ctypes.data_as(_lib._dp)

    def AddDomainIntegral(self, kind, params=None):
        _lib.call("sfx_qoi_add_domain_integral", self._h, int(kind), self._params(kind, params, False))

    def AddBoundaryIntegral(self, kind, sides=None, params=None, faces=None):
        prm = self._params(kind, params, True)
        if faces is not None:
            e, s2 = _face_arrays(faces)
            self._keep += [e, s2]
            _lib.call("sfx_qoi_add_boundary_integral_faces", self._h, int(kind), ctypes.c_int64(e.size),
                      e.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), s2.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                      prm)
            return
        mask = 0
        for s_ in sides:
            mask |= 1 << (s_ - 1)
        _lib.call("sfx_qoi_add_boundary_integral", self._h, int(kind), mask, prm)

    AddVolumeIntegral = AddDomainIntegral
    AddSurfaceIntegral = AddBoundaryIntegral

    def set_shape_displacement(self, shape, stream=None):
        """Evaluate on the configuration X + shape (as Functional.set_shape_displacement)."""
        if shape is None:
            _lib.call("sfx_form_set_shape_displacement", self._h, None, _stream(stream))
        else:
            _require(shape, torch.float64, 3 * self.num_nodes, "shape")
            _lib.call("sfx_form_set_shape_displacement", self._h, _dptr(shape), _stream(stream))

    def shape_gradient(self, t, u, out=None, stream=None):
        """dQ/dp (3 * num_nodes): the partial derivative with respect to the
        shape displacement at the current shape."""
        _require(u, torch.float64, self.ndofs, "u")
        out = torch.empty(3 * self.num_nodes, dtype=torch.float64, device=u.device) if out is None else out
        _lib.call("sfx_qoi_shape_gradient", self._h, float(t), _dptr(u), _dptr(out), _stream(stream))
        return out

    def value(self, t, u, out=None, stream=None):
        """Q(t, u) as a one-element float64 CUDA tensor (no host synchronisation)."""
        _require(u, torch.float64, self.ndofs, "u")
        out = torch.empty(1, dtype=torch.float64, device=u.device) if out is None else out
        _lib.call("sfx_qoi_evaluate", self._h, float(t), _dptr(u), _dptr(out), _stream(stream))
        return out

    def gradient(self, t, u, out=None, value=None, stream=None):
        """dQ/du (t, u) as a CUDA tensor; value (one-element tensor) receives Q."""
        _require(u, torch.float64, self.ndofs, "u")
        out = torch.empty_like(u) if out is None else out
        _lib.call("sfx_qoi_gradient", self._h, float(t), _dptr(u), _dptr(value), _dptr(out), _stream(stream))
        return out

    def __call__(self, t, arg):
        if isinstance(arg, differentiate_wrt):
            return float(self.value(t, arg.u).item()), QoIGradient(self, t, arg.u)
        return float(self.value(t, arg).item())


PARAM_NEOHOOKEAN = 16  # multi-field: (displacement 3, acceleration 3, dK 1, dG 1), params {density, K0, G0}
_MULTI_ARGS = {PARAM_NEOHOOKEAN: (3, 3, 1, 1)}


class MultiGradient:
    """dR/d(field wrt) at the linearisation point of a MultiFunctional:
    mult(d) applies it to a direction of that field, mult_transpose(v) maps a
    test-space vector onto the field (functional.hpp:534-708 for one argument)."""

    def __init__(self, form, wrt):
        self.form, self.wrt = form, wrt

    def mult(self, d, out=None, stream=None):
        f = self.form
        _require(d, torch.float64, f.components[self.wrt] * f.num_nodes, "direction")
        out = torch.empty(f.ndofs, dtype=torch.float64, device=d.device) if out is None else out
        _lib.call("sfx_mform_jvp", f._h, self.wrt, _dptr(d), _dptr(out), _stream(stream))
        return out

    Mult = mult
    __call__ = mult

    def mult_transpose(self, v, out=None, stream=None):
        f = self.form
        _require(v, torch.float64, f.ndofs, "v")
        n = f.components[self.wrt] * f.num_nodes
        out = torch.empty(n, dtype=torch.float64, device=v.device) if out is None else out
        _lib.call("sfx_mform_jvp_transpose", f._h, self.wrt, _dptr(v), _dptr(out), _stream(stream))
        return out

    MultTranspose = mult_transpose


class MultiFunctional:
    """Functional<test(trial_0, ..., trial_{n-1})> (functional.hpp:189-317) on a
    structured hex mesh: every trial space H1 of the test space's order on the
    same node grid, with its own component count; SolidMechanics' residual is
    MultiFunctional(mesh, H1(p, 3), [H1(p, 3), H1(p, 3), H1(p, 1), H1(p, 1)])
    for (displacement, acceleration, two parameter fields).

        f.AddDomainIntegral(PARAM_NEOHOOKEAN, depends_on=[0, 1, 2, 3], params=[rho, K0, G0])
        r = f(t, u, a, dK, dG)
        r, dR_ddK = f(t, u, a, differentiate_wrt(dK), dG)
        dR_ddK.mult(ddK); dR_ddK.mult_transpose(lam)
    """

    def __init__(self, mesh, test: H1, trials):
        self.mesh = mesh
        self.test = test
        self.trials = list(trials)
        if any(t.order != test.order for t in self.trials):
            raise ValueError("every trial space must have the test space's order")
        self.components = [t.components for t in self.trials]
        comps = (ctypes.c_int * len(self.components))(*self.components)
        h = ctypes.c_void_p()
        _lib.call("sfx_mform_create", mesh._h, test.order, test.components, len(self.components), comps,
                  ctypes.byref(h))
        self._h = h
        n = ctypes.c_int64()
        _lib.call("sfx_mform_num_nodes", h, ctypes.byref(n))
        self.num_nodes = n.value
        self.ndofs = self.num_nodes * test.components

    def __del__(self):
        if getattr(self, "_h", None) and _lib._LIB is not None:
            _lib.load().sfx_mform_destroy(self._h)
            self._h = None

    def AddDomainIntegral(self, material, depends_on, params, per_element=False):
        dep = (ctypes.c_int * len(depends_on))(*depends_on)
        arr = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
        _lib.call("sfx_mform_add_domain_integral", self._h, int(material), dep, len(depends_on),
                  arr.ctypes.data_as(_lib._dp), int(bool(per_element)))

    def _fields(self, fields):
        if len(fields) != len(self.components):
            raise ValueError(f"expected {len(self.components)} fields")
        ptrs = (ctypes.c_void_p * len(fields))()
        for i, (u, c) in enumerate(zip(fields, self.components)):
            _require(u, torch.float64, c * self.num_nodes, f"field {i}")
            ptrs[i] = u.data_ptr()
        return ptrs

    def residual(self, t, fields, out=None, stream=None):
        out = torch.empty(self.ndofs, dtype=torch.float64, device=fields[0].device) if out is None else out
        _lib.call("sfx_mform_residual", self._h, float(t), self._fields(fields), _dptr(out), _stream(stream))
        return out

    def linearize(self, t, fields, wrt, stream=None):
        _lib.call("sfx_mform_linearize", self._h, float(t), self._fields(fields), int(wrt), _stream(stream))
        return MultiGradient(self, wrt)

    def __call__(self, t, *args):
        wrt = [i for i, a in enumerate(args) if isinstance(a, differentiate_wrt)]
        fields = [a.u if isinstance(a, differentiate_wrt) else a for a in args]
        r = self.residual(t, fields)
        if not wrt:
            return r
        if len(wrt) > 1:
            raise ValueError("differentiate with respect to one argument at a time")
        return r, self.linearize(t, fields, wrt[0])


def assemble(gradient):
    """CSR of dR/du at the linearisation point, (row_ptr int64, col int32,
    values float64); for a QoI gradient, the vector dQ/du."""
    if isinstance(gradient, QoIGradient):
        return gradient.assemble()
    f = gradient.form
    row_ptr, col = f.csr_graph()
    return row_ptr, col, f.assemble_values()
