"""Lowest-order Nedelec H(curl) on affine tetrahedra
(python/skfemntv/hcurl_basis.py:292-445, hcurl_assembler.py:52-215,
edge_topology.py, edge_dof_map.py).

Edge numbering, orientation signs and the Maxwell assembly run on the GPU.
The mapped per-point basis arrays the reference keeps, ``(E, 6, 3, Q)`` for
values and curls, are not stored; they are produced on demand by the
``values`` / ``curls`` properties for callers that read them.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _device as dev
from . import quadrature as quad
from ._native import SKG_FP64, call
from .assembly import Pattern, _MatrixTarget, _precision, per_element, per_point
from .mesh import oriented_edges
from .preflight import enforce_memory_budget, estimate_n1_memory


@dataclass(frozen=True)
class OrientedEdgeTopology:
    edges: np.ndarray
    element_edges: np.ndarray
    element_edge_signs: np.ndarray
    local_edges: tuple


@dataclass(frozen=True)
class OrientedEdgeDofMap:
    topology: OrientedEdgeTopology

    @property
    def ndofs(self):
        return int(self.topology.edges.shape[1])

    @property
    def element_dofs(self):
        return self.topology.element_edges

    @property
    def basis_signs(self):
        return self.topology.element_edge_signs

    def local_coefficients(self, global_coefficients):
        """Global edge moments (n_edges,) to coefficients of the oriented local
        bases, (6, E) (edge_dof_map.py:34-41)."""
        values = np.asarray(global_coefficients)
        if values.ndim != 1 or values.shape[0] != self.ndofs:
            raise ValueError(f"global edge coefficients must have shape ({self.ndofs},)")
        return self.basis_signs * values[self.element_dofs]

    def global_moments_from_local(self, local_coefficients):
        """Per-cell global-oriented moments from local coefficients (6, E),
        cells not merged (edge_dof_map.py:43-51)."""
        values = np.asarray(local_coefficients)
        if values.shape != self.element_dofs.shape:
            raise ValueError(f"local edge coefficients must have shape {self.element_dofs.shape}")
        return self.basis_signs * values


def build_oriented_edge_topology(mesh):
    """Global edges of a tetrahedral mesh's corners, numbered first-seen in
    cell-major, local-edge-major order with ascending vertex pairs, and the
    sign of each directed local edge against its global one
    (edge_topology.py:33-63), computed on the device.  Edge nodes of a
    quadratic mesh do not change edge identity."""
    if int(mesh.dim()) != 3:
        raise NotImplementedError("oriented edge topology supports tetrahedra")
    if mesh.t.shape[0] < 4:
        raise ValueError("mesh connectivity does not contain all corner vertices")
    if hasattr(mesh, "_dev"):
        t4 = mesh._dev("t")[:4].contiguous()
    else:  # any object with a connectivity ``t`` and ``dim()``
        t4 = dev.to_device(np.asarray(mesh.t)[:4], np.int32)
    edges, ee, sg = oriented_edges(t4, int(t4.shape[1]))
    return OrientedEdgeTopology(edges, ee.cpu().numpy().astype(np.int64), sg.cpu().numpy(), quad.TET_EDGES)


def build_oriented_edge_dof_map(mesh):
    """One scalar DOF per global edge (edge_dof_map.py:54-55)."""
    return OrientedEdgeDofMap(build_oriented_edge_topology(mesh))


@dataclass(frozen=True)
class HcurlTetGeometryDiagnostics:
    minimum_signed_determinant: float
    minimum_absolute_determinant: float
    minimum_volume: float
    maximum_aspect_ratio: float
    inverted_cell_count: int


def _ref_basis(X):
    lam = np.concatenate(((1.0 - X.sum(axis=0))[None], X), axis=0)
    g = quad._DL
    vals = np.empty((6, 3) + X.shape[1:])
    for k, (a, b) in enumerate(quad.TET_EDGES):
        vals[k] = lam[a][None] * g[b][:, None] - lam[b][None] * g[a][:, None]
    curls = np.array([2.0 * np.cross(g[a], g[b]) for a, b in quad.TET_EDGES])
    return vals, curls


class AffineTetN1Basis:
    """Lowest-order H(curl) basis on affine tetrahedral meshes."""

    def __init__(self, mesh, *, intorder=2, max_aspect_ratio=None):
        if mesh.dim() != 3 or mesh.t.shape[0] not in (4, 10):
            raise TypeError("AffineTetN1Basis requires a tetrahedral mesh")
        self.mesh = mesh
        E = mesh.nelements
        t4 = mesh._dev("t")[:4].contiguous()
        edges, ee, sg = oriented_edges(t4, E)
        self._t4 = t4
        self._ee_dev, self._signs_dev = ee, sg
        topo = OrientedEdgeTopology(edges, ee.cpu().numpy().astype(np.int64), sg.cpu().numpy(),
                                    quad.TET_EDGES)
        self.dof_map = OrientedEdgeDofMap(topo)
        self.N = self.dof_map.ndofs
        self.element_dofs = self.dof_map.element_dofs
        self.basis_signs = self.dof_map.basis_signs
        self.X, self.W = quad.duffy_rule(intorder)
        v = mesh.p[:, mesh.t[:4]]
        self.jacobians = np.stack(tuple(v[:, k] - v[:, 0] for k in (1, 2, 3)), axis=1)
        J = self.jacobians
        self.detJ = (J[0, 0] * (J[1, 1] * J[2, 2] - J[1, 2] * J[2, 1])
                     - J[0, 1] * (J[1, 0] * J[2, 2] - J[1, 2] * J[2, 0])
                     + J[0, 2] * (J[1, 0] * J[2, 1] - J[1, 1] * J[2, 0]))
        if np.any(np.isclose(self.detJ, 0.0)):
            raise ValueError("H(curl) basis requires nonsingular tetrahedra")
        lengths = [np.linalg.norm(v[:, b] - v[:, a], axis=0) for a, b in quad.TET_EDGES]
        aspect = np.max(lengths, axis=0) ** 3 / np.abs(self.detJ)
        self.geometry_diagnostics = HcurlTetGeometryDiagnostics(
            minimum_signed_determinant=float(np.min(self.detJ)),
            minimum_absolute_determinant=float(np.min(np.abs(self.detJ))),
            minimum_volume=float(np.min(np.abs(self.detJ)) / 6.0),
            maximum_aspect_ratio=float(np.max(aspect)),
            inverted_cell_count=int(np.count_nonzero(self.detJ < 0.0)))
        if max_aspect_ratio is not None:
            if (isinstance(max_aspect_ratio, bool) or not np.isscalar(max_aspect_ratio)
                    or not np.isfinite(max_aspect_ratio) or max_aspect_ratio <= 0.0):
                raise ValueError("max_aspect_ratio must be a positive finite scalar")
            if self.geometry_diagnostics.maximum_aspect_ratio > max_aspect_ratio:
                raise ValueError(
                    f"H(curl) tetrahedron aspect ratio exceeds max_aspect_ratio={max_aspect_ratio}")
        self.dx = np.abs(self.detJ)[:, None] * self.W[None, :]

    def _mapped(self):
        ref_v, ref_c = _ref_basis(self.X)
        J = np.moveaxis(self.jacobians, (0, 1), (-2, -1))  # (E,3,3)
        inv = np.linalg.inv(J)
        vals = np.einsum("erp,brq->ebpq", inv, ref_v)
        curls = np.einsum("epr,br->ebp", J, ref_c)[..., None] / self.detJ[:, None, None, None]
        curls = np.broadcast_to(curls, vals.shape)
        s = self.basis_signs.T[:, :, None, None]
        return vals * s, curls * s

    @property
    def global_coordinates(self):
        """Physical quadrature coordinates as (component, cell, point) (hcurl_basis.py:435-440)."""
        vertices = self.mesh.p[:, self.mesh.t[0]]
        return vertices[:, :, None] + np.einsum("ire,rq->ieq", self.jacobians, self.X)

    @property
    def values(self):
        """Mapped values as (basis, component, cell, quadrature)."""
        return self._mapped()[0].transpose(1, 2, 0, 3)

    @property
    def curls(self):
        return self._mapped()[1].transpose(1, 2, 0, 3)

    # ------------------------------------------------------------ device evaluation
    def _element_matrices(self, include_mass, include_curl):
        E, Q = self.dx.shape
        out = dev.empty((E, 6, 6), np.float64)
        call("skg_n1_element_matrices", dev.ptr(self.mesh._dev("p")), self.mesh.p.shape[1], dev.ptr(self._t4),
             dev.ptr(self._signs_dev), E, Q, dev.hptr(self.X), dev.hptr(self.W), None, None, 0,
             int(include_mass), int(include_curl), dev.ptr(out), dev.stream_ptr())
        return out.cpu().numpy()

    def element_mass_matrices(self):
        """(E, 6, 6) element mass matrices sum_q dx v_a . v_c
        (hcurl_basis.py:376-380), computed on the device."""
        return self._element_matrices(True, False)

    def element_curl_curl_matrices(self):
        """(E, 6, 6) element curl-curl matrices sum_q dx c_a . c_c
        (hcurl_basis.py:382-386), computed on the device."""
        return self._element_matrices(False, True)

    def _edges_device(self):
        if not hasattr(self, "_edges_dev"):
            self._edges_dev = dev.to_device(self.dof_map.topology.edges, np.int32)  # (2, n_edges)
        return self._edges_dev

    def interpolate_edge_moments(self, field, *, quadrature_order=4):
        """Interpolate a vector field by tangential moments along the
        ascending global edges (hcurl_basis.py:388-416): for edge (a, b),
        m = sum_q w_q field(x_q) . (p_b - p_a) on the Gauss-Legendre rule of
        ``quadrature_order`` points mapped to the edge.  The points are made
        and the moments summed on the device; ``field`` is called once, with
        the points of every edge as one (3, n_edges * order) array, edge-major
        (the reference calls it once per edge with (3, order))."""
        if not callable(field):
            raise TypeError("field must be callable")
        if (isinstance(quadrature_order, bool) or not isinstance(quadrature_order, (int, np.integer))
                or quadrature_order < 1):
            raise ValueError("quadrature_order must be a positive integer")
        nodes, weights = np.polynomial.legendre.leggauss(int(quadrature_order))
        param = np.ascontiguousarray(0.5 * (nodes + 1.0))
        weights = np.ascontiguousarray(0.5 * weights)
        n_edges, nq = self.N, len(param)
        p, npts = dev.ptr(self.mesh._dev("p")), self.mesh.p.shape[1]
        edges = dev.ptr(self._edges_device()) if n_edges else None
        points = dev.empty((3, n_edges * nq), np.float64)
        call("skg_n1_edge_points", p, npts, edges, n_edges, nq, dev.hptr(param), dev.ptr(points), dev.stream_ptr())
        x = points.cpu().numpy()
        values = np.asarray(field(x), dtype=np.float64)
        try:
            values = np.broadcast_to(values, x.shape)
        except ValueError as error:
            raise ValueError("field must return vectors broadcastable to (3, points)") from error
        d_values = dev.to_device(values, np.float64)
        out = dev.empty(max(1, n_edges), np.float64)
        call("skg_n1_edge_moments", p, npts, edges, n_edges, nq, dev.hptr(weights), dev.ptr(d_values),
             dev.ptr(out), dev.stream_ptr())
        return out[:n_edges].cpu().numpy()

    def _evaluate(self, coefficients, curl):
        u = np.asarray(coefficients, dtype=np.float64)
        if u.shape != (self.N,):
            raise ValueError(f"coefficients must have shape ({self.N},)")
        E, Q = self.dx.shape
        out = dev.empty((3, E, Q), np.float64)
        d_u = dev.to_device(u, np.float64)
        call("skg_n1_evaluate", dev.ptr(self.mesh._dev("p")), self.mesh.p.shape[1], dev.ptr(self._t4),
             dev.ptr(self._ee_dev), dev.ptr(self._signs_dev), E, self.N, Q, dev.hptr(self.X), dev.ptr(d_u),
             int(curl), dev.ptr(out), dev.stream_ptr())
        return out.cpu().numpy()

    def evaluate(self, coefficients):
        """A global edge field at the rule's points, (component, cell, point)
        (hcurl_basis.py:424-427), computed on the device."""
        return self._evaluate(coefficients, False)

    def evaluate_curl(self, coefficients):
        """Its vector curl, (component, cell, point) (hcurl_basis.py:429-432),
        computed on the device."""
        return self._evaluate(coefficients, True)


def estimate_tet_n1_assembly_memory(basis):
    if not isinstance(basis, AffineTetN1Basis):
        raise TypeError("basis must be AffineTetN1Basis")
    return estimate_n1_memory(basis, basis.mesh.nelements, len(basis.W), int(basis.N))


class TetN1Assembler:
    """Reusable mass / curl-curl assembler; assembly methods overwrite and
    return one CSR matrix (call ``.copy()`` to keep a result)."""

    def __init__(self, basis, *, memory_limit_bytes=None, memory_safety_factor=1.25):
        if not isinstance(basis, AffineTetN1Basis):
            raise TypeError("basis must be AffineTetN1Basis")
        self.basis = basis
        self.memory_estimate = estimate_tet_n1_assembly_memory(basis)
        enforce_memory_budget(self.memory_estimate, memory_limit_bytes, safety_factor=memory_safety_factor)
        E = basis.mesh.nelements
        self._dofs = basis._ee_dev.t().contiguous()  # (E, 6)
        self.pattern = Pattern(self._dofs, self._dofs, E, 6, 6, basis.N, basis.N)
        self.target = _MatrixTarget(self.pattern, (basis.N, basis.N))
        self._keep = None

    def _coef(self, name, value):
        """(per-element values (host array) or None, per-point device array or
        None); per-element values of 1 are dropped (the kernels' default)."""
        E, Q = self.basis.dx.shape
        if value is None:
            return None, None
        pe = per_element(value, E, Q, name)
        if pe is not None:
            if np.ndim(pe) == 0:  # scalar: none for 1 (the kernels' default)
                return (None if float(pe) == 1.0 else np.full(E, float(pe))), None
            return np.ascontiguousarray(pe, dtype=np.float64), None
        return None, dev.to_device(per_point(value, E, Q, name), np.float64)

    def _element_pointer(self, pe, host, keep):
        """Kernel pointer of per-element values: read in place from host memory
        on the host-output path when the device can, else uploaded."""
        if pe is None:
            return None
        if host:
            ptr = dev.host_readable(pe)
            if ptr is not None:
                keep.append(pe)
                return ptr
        d = dev.to_device(pe, np.float64)
        keep.append(d)
        return dev.ptr(d)

    def assemble_device(self, *, mass_coefficient=None, curl_coefficient=None, include_mass=True,
                        include_curl=True, precision="fp64", _out=None):
        """Assemble into the device values (with ``_out``, the host matrix's
        page-locked values, also into those); returns the device values tensor.
        The caller synchronises before host arrays passed in go away."""
        b = self.basis
        d_values = dev.ptr(self.target.d_values)
        E = b.mesh.nelements
        Q = len(b.W)
        prec = _precision(precision)
        m_el, m_pt = self._coef("mass", mass_coefficient)
        c_el, c_pt = self._coef("curl", curl_coefficient)
        keep = []
        if m_pt is None and c_pt is None:
            args = (self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1], dev.ptr(b._t4),
                    dev.ptr(b._ee_dev), dev.ptr(b._signs_dev), E, Q, dev.hptr(b.X), dev.hptr(b.W),
                    self._element_pointer(m_el, _out is not None, keep),
                    self._element_pointer(c_el, _out is not None, keep), int(include_mass), int(include_curl),
                    prec, d_values)
            if _out is not None:
                call("skg_n1_assemble_host", *args, _out, dev.stream_ptr())
            else:
                call("skg_n1_assemble", *args, dev.stream_ptr())
            self._keep = keep
        else:
            if prec != SKG_FP64:
                from .errors import UnsupportedNativeForm

                raise UnsupportedNativeForm("split precision needs per-element coefficients")
            ones = dev.to_device(np.ones((E, Q)), np.float64)
            mp = m_pt if m_pt is not None else (
                ones if m_el is None else dev.to_device(np.repeat(m_el[:, None], Q, 1), np.float64))
            cp = c_pt if c_pt is not None else (
                ones if c_el is None else dev.to_device(np.repeat(c_el[:, None], Q, 1), np.float64))
            call("skg_n1_assemble_pointwise", self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1],
                 dev.ptr(b._t4), dev.ptr(b._signs_dev), E, Q, dev.hptr(b.X), dev.hptr(b.W), dev.ptr(mp),
                 dev.ptr(cp), int(include_mass), int(include_curl), d_values, dev.stream_ptr())
            if _out is not None:
                self.target.enqueue_download()
        return self.target.d_values

    def _host(self, **kw):
        """Host matrix: the values are copied chunk by chunk into its
        page-locked buffer while the later chunks are computed."""
        self.assemble_device(_out=self.target.pinned_ptr(), **kw)
        out = self.target.finish_direct()
        self._keep = None
        return out

    def assemble_maxwell_torch(self, *, mass_coefficient=None, curl_coefficient=None, precision="fp64"):
        """Device-resident Maxwell matrix: a CUDA sparse CSR tensor (values reused)."""
        self.assemble_device(mass_coefficient=mass_coefficient, curl_coefficient=curl_coefficient,
                             precision=precision)
        return self.target.torch_csr()

    def assemble_maxwell(self, *, mass_coefficient=None, curl_coefficient=None, precision="fp64"):
        return self._host(mass_coefficient=mass_coefficient, curl_coefficient=curl_coefficient, precision=precision)

    def assemble_mass(self, coefficient=None, precision="fp64"):
        return self._host(mass_coefficient=coefficient, include_curl=False, precision=precision)

    def assemble_curl_curl(self, coefficient=None, precision="fp64"):
        return self._host(curl_coefficient=coefficient, include_mass=False, precision=precision)


class TetN1LinearAssembler:
    """Reusable vector-load assembler for ``AffineTetN1Basis``
    (hcurl_assembler.py:218-266): ``assemble_vector_load(field)`` returns the
    reused load vector r_a = int f . phi_a."""

    def __init__(self, basis):
        if not isinstance(basis, AffineTetN1Basis):
            raise TypeError("basis must be AffineTetN1Basis")
        self.basis = basis
        E = basis.mesh.nelements
        self._dofs = basis._ee_dev.t().contiguous()  # (E, 6)
        self.pattern = Pattern(self._dofs, None, E, 6, 0, basis.N, 0)
        self._vector = np.zeros(basis.N, dtype=np.float64)
        self._d_out = dev.empty(max(1, basis.N), np.float64)

    def _values(self, field):
        b = self.basis
        values = field(b.global_coordinates) if callable(field) else field
        values = np.asarray(values, dtype=np.float64)
        expected = (3,) + b.dx.shape
        try:
            return np.broadcast_to(values, expected)
        except ValueError as error:
            raise ValueError(f"vector load must broadcast to {expected}") from error

    def assemble_vector_load(self, field):
        b = self.basis
        E, Q = b.dx.shape
        f = dev.to_device(self._values(field), np.float64)
        call("skg_n1_vector_load", self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1], dev.ptr(b._t4),
             dev.ptr(b._signs_dev), E, Q, dev.hptr(b.X), dev.hptr(b.W), dev.ptr(f), dev.ptr(self._d_out),
             dev.stream_ptr())
        self._vector[:] = self._d_out[: b.N].cpu().numpy()
        return self._vector
