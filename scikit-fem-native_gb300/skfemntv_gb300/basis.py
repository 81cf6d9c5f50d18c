"""Nodal H1 basis on tetrahedra (python/skfemntv/basis.py:1620-1800, 2194-2356).

Host side (as in the reference): quadrature selection, active-node
compaction and DOF numbering (DOF = node position * components + component,
element_dofs node-major then component).  Device side: the per-(element,
point) geometry is computed by the GPU kernel behind
``skg_tabulate_geometry``, which also validates the mesh exactly as the
reference does at construction (same error messages).  The large tabulated
arrays (``tabulated_gradients``, ``dx``, ...) are produced on the device only
when something asks for them; the fused affine assembly never needs them.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _device as dev
from . import quadrature as quad
from ._native import call
from .element import ElementTetP1, ElementTetP2, ElementVector


# The geometry kernel keeps the rule's reference tables (values and gradients
# of the element and geometry nodes, weights) in one block's shared memory,
# at most 227 KB on sm_103a: up to 343 points for P2 (order 11 and below).
_GEOMETRY_TABLE_BYTES = 227 * 1024


@dataclass(frozen=True)
class GeometryDiagnostics:
    element_count: int
    quadrature_points_per_element: int
    minimum_determinant: float
    maximum_determinant: float
    minimum_scaled_determinant: float
    worst_element: int
    worst_quadrature_point: int
    determinant_tolerance: float
    negative_orientation_elements: int
    maximum_condition_number: float
    worst_condition_element: int
    worst_condition_quadrature_point: int


def number_dofs(n_points, conn, comp):
    """Active-node compaction and DOF numbering (basis.py:1749-1777).

    Returns (N, nodal_dofs (comp, n_active), element_dofs (nodes*comp, E),
    active node ids)."""
    nodes, E = conn.shape
    used = np.zeros(n_points, dtype=bool)
    used[conn] = True
    active = np.flatnonzero(used)
    N = len(active) * comp
    nodal_dofs = np.arange(N).reshape(-1, comp).T
    pos = np.full(n_points, -1, dtype=np.int64)
    pos[active] = np.arange(len(active))
    local = pos[conn]
    element_dofs = nodal_dofs[:, local].transpose(2, 1, 0).reshape(E, nodes * comp).T
    return N, nodal_dofs, element_dofs, active


class Basis:
    def __init__(self, mesh, element, intorder=2, quadrature=None, elements=None):
        if elements is not None:
            from .errors import UnsupportedNativeForm

            raise UnsupportedNativeForm("element restriction is not supported by the GPU backend")
        intorder = 2 if intorder is None else int(intorder)
        self.intorder = intorder
        scalar = element.elem if isinstance(element, ElementVector) else None
        if not isinstance(element, ElementVector) or not isinstance(scalar, (ElementTetP1, ElementTetP2)):
            raise NotImplementedError("independent Basis supports P0 and nodal H1/DG elements")
        self.mesh, self.elem = mesh, element
        self._quadratic = isinstance(scalar, ElementTetP2)
        self._nodes = 10 if self._quadratic else 4
        self._comp = element._dim
        if quadrature is not None:
            self.X, self.W = quad.validate(quadrature, 3)
        elif intorder > 4:
            self.X, self.W = quad.simplex_rule(intorder)
        elif self._quadratic or intorder >= 4:
            self.X, self.W = quad.tet_rule_p2()
        else:
            self.X, self.W = quad.tet_rule_p1()
        self.quadrature = (self.X.copy(), self.W.copy())
        G = mesh.t.shape[0]
        if G < self._nodes:
            raise ValueError("mesh geometry nodes are incompatible with the element")
        table_bytes = 8 * len(self.W) * (4 * self._nodes + 4 * G + 1)
        if table_bytes > _GEOMETRY_TABLE_BYTES:
            from .errors import UnsupportedNativeForm

            raise UnsupportedNativeForm(
                f"a rule of {len(self.W)} points needs {table_bytes} bytes of reference tables; the geometry "
                f"kernel holds at most {_GEOMETRY_TABLE_BYTES} in shared memory")
        conn = mesh.t[: self._nodes]
        E = mesh.nelements
        C = self._comp
        self.N, self.nodal_dofs, self.element_dofs, active = number_dofs(mesh.p.shape[1], conn, C)
        self.doflocs = np.repeat(mesh.p[:, active], C, axis=1)
        self.active_nodes = active
        self.field_connectivity = conn
        self.tind = np.arange(E, dtype=np.int64)
        self.normals = None
        self._tab = None
        self._tab_host = {}
        self._validate_geometry()

    # ------------------------------------------------------------ tables
    def _tables(self):
        shape, refgrad = quad.tabulate(self.X, self._quadratic)
        if self.mesh.t.shape[0] != self._nodes:
            gshape, gref = quad.tabulate(self.X, True)
        else:
            gshape, gref = shape, refgrad
        return [np.ascontiguousarray(a, dtype=np.float64) for a in (shape, refgrad, gshape, gref, self.W)]

    def _run_tabulation(self, outputs):
        E, Q = self.mesh.nelements, len(self.W)
        tabs = self._tables()
        bad = (ctypes.c_int64 * 3)()
        call("skg_tabulate_geometry", dev.ptr(self.mesh._dev("p")), self.mesh.p.shape[1],
             dev.ptr(self.mesh._dev("t")), self.mesh.t.shape[0], E, Q, self._nodes,
             *(dev.hptr(a) for a in tabs),
             *(dev.ptr(outputs.get(k)) for k in ("shape", "grad", "dx", "x", "det", "tol", "cond")),
             bad, dev.stream_ptr())

    def _validate_geometry(self):
        E, Q = self.mesh.nelements, len(self.W)
        out = {k: dev.empty((E, Q), np.float64) for k in ("det", "tol", "cond")}
        self._run_tabulation(out)
        self._geom = out

    def _device_tabulation(self):
        """Device tensors shape (E,Q,n), grad (E,Q,n,3), dx (E,Q), x (E,Q,3)."""
        if self._tab is None:
            E, Q, n = self.mesh.nelements, len(self.W), self._nodes
            out = {
                "shape": dev.empty((E, Q, n), np.float64),
                "grad": dev.empty((E, Q, n, 3), np.float64),
                "dx": dev.empty((E, Q), np.float64),
                "x": dev.empty((E, Q, 3), np.float64),
                "det": dev.empty((E, Q), np.float64),
                "tol": dev.empty((E, Q), np.float64),
                "cond": dev.empty((E, Q), np.float64),
            }
            self._run_tabulation(out)
            self._tab = out
        return self._tab

    def _host(self, key):
        if key not in self._tab_host:
            self._tab_host[key] = self._device_tabulation()[key].cpu().numpy()
        return self._tab_host[key]

    @property
    def tabulated_shape(self):
        return self._host("shape")

    @property
    def tabulated_gradients(self):
        return self._host("grad")

    @property
    def dx(self):
        return self._host("dx")

    @property
    def global_coordinates(self):
        return self._host("x")

    @property
    def nelems(self):
        """Number of elements (basis.py:1804-1806), from the mesh: reading dx
        would make the device tabulation."""
        return int(self.mesh.nelements)

    @property
    def _coefficient_shape(self):
        return (self.mesh.nelements, len(self.W))

    @property
    def _geometry_determinants(self):
        return self._geom["det"].cpu().numpy()

    @property
    def _geometry_tolerances(self):
        return self._geom["tol"].cpu().numpy()

    @property
    def _geometry_condition_numbers(self):
        return self._geom["cond"].cpu().numpy()

    @property
    def geometry_diagnostics(self):
        """Same fields and selection rules as basis.py:2296-2356, reduced on the
        device (skg_geometry_diagnostics): nothing of size (E, Q) is copied."""
        det = self._geom["det"]
        E, Q = (int(det.shape[0]), int(det.shape[1])) if det.dim() == 2 else (0, 0)
        if E == 0 or Q == 0:
            return GeometryDiagnostics(0, Q, float("inf"), float("-inf"), float("inf"), -1, -1, 0.0, 0, 0.0, -1, -1)
        vals = np.empty(4, dtype=np.float64)
        idx = np.empty(3, dtype=np.int64)
        call("skg_geometry_diagnostics", dev.ptr(det), dev.ptr(self._geom["tol"]), dev.ptr(self._geom["cond"]),
             E, Q, dev.hptr(vals), dev.hptr(idx), dev.stream_ptr())
        e, q = divmod(int(idx[0]), Q)
        ce, cq = divmod(int(idx[1]), Q)
        tol = float(self._geom["tol"].view(-1)[int(idx[0])].item())
        return GeometryDiagnostics(
            element_count=E, quadrature_points_per_element=Q,
            minimum_determinant=float(vals[0]), maximum_determinant=float(vals[1]),
            minimum_scaled_determinant=float(vals[2]), worst_element=e,
            worst_quadrature_point=q, determinant_tolerance=tol,
            negative_orientation_elements=int(idx[2]),
            maximum_condition_number=float(vals[3]), worst_condition_element=ce,
            worst_condition_quadrature_point=cq)

    # ------------------------------------------------------------ device maps
    def _dev_dofs(self):
        if not hasattr(self, "_dofs_dev"):
            self._dofs_dev = dev.to_device(self.element_dofs.T, np.int32)  # (E, L)
        return self._dofs_dev

    @property
    def is_affine(self):
        """True when every element map is affine (P1 geometry, or P2 edge
        nodes at the midpoints of their edges)."""
        if not hasattr(self, "_affine"):
            t = self.mesh.t
            if t.shape[0] == 4:
                self._affine = True
            else:
                p = self.mesh.p
                scale = max(1.0, float(np.max(np.abs(p)))) if p.size else 1.0
                ok = True
                for k, (a, b) in enumerate(quad.TET_EDGES):
                    mid = 0.5 * (p[:, t[a]] + p[:, t[b]])
                    if np.max(np.abs(p[:, t[4 + k]] - mid), initial=0.0) > 1e-14 * scale:
                        ok = False
                        break
                self._affine = ok
        return self._affine
