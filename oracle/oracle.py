"""CPU oracle for the finite-element assembly hot path (test infrastructure).

This module is the checker used by ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg; the GPU backend never imports it.  It
restates the reference package's (scikit-fem-native ``skfemntv`` 0.3.1)
pipeline for the hot path:

* numpy restatements of the reference's Python setup layer (mesh generation,
  P2 edge nodes, quadrature rules, reference-basis tabulation, DOF numbering,
  the Nedelec N1 mapping chain, the neo-Hookean law), each citing its source;
* ctypes calls into ``fem_oracle.c`` for the reference's C++ kernels
  (geometry tabulation, CSR pattern, bilinear/cross/linear assembly, edge
  topology, N1 integration).

The oracle is pinned against outputs of the reference itself: the fixtures
under ``tests/golden`` were generated by ``tests/golden/make_golden.py`` with
the real reference, and ``tests/test_oracle_golden.py`` checks the oracle
against every one of them.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfem_oracle.so")
_lib = None

_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_I64 = ctypes.c_int64
_INT = ctypes.c_int


def build(quiet: bool = True) -> str:
    """Compile ``fem_oracle.c`` with the committed Makefile."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
        os.path.join(_HERE, "fem_oracle.c")
    ):
        build()
    L = ctypes.CDLL(_LIB_PATH)
    L.fo_max_threads.restype = _INT
    L.fo_tabulate_geometry.restype = _INT
    L.fo_tabulate_geometry.argtypes = [
        _INT, _I64, _f64p, _I64, _I64, _i64p, _I64, _I64, _f64p, _f64p, _f64p, _f64p, _f64p,
        _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, _INT,
        ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_INT),
    ]
    L.fo_pattern_build.restype = _vp
    L.fo_pattern_build.argtypes = [_i64p, _i64p, _I64, _I64, _I64, _I64, _INT]
    L.fo_pattern_free.argtypes = [_vp]
    for name in ("fo_pattern_nnz", "fo_pattern_nrows", "fo_pattern_ncolors"):
        getattr(L, name).restype = _I64
        getattr(L, name).argtypes = [_vp]
    L.fo_pattern_copy.argtypes = [_vp, _vp, _vp, _vp]
    L.fo_bilinear_assemble.restype = _INT
    L.fo_bilinear_assemble.argtypes = [
        _vp, _I64, _I64, _I64, _I64, _f64p, _f64p, _f64p, _vp, _vp, _vp, _vp, _INT, _f64p,
    ]
    L.fo_cross_assemble.restype = _INT
    L.fo_cross_assemble.argtypes = [
        _vp, _I64, _I64, _I64, _I64, _I64, _I64, _I64, _f64p, _f64p, _vp, _vp, _f64p, _vp,
        _INT, _INT, _INT, _INT, _f64p,
    ]
    L.fo_linear_assemble.restype = _INT
    L.fo_linear_assemble.argtypes = [
        _i64p, _I64, _I64, _I64, _I64, _I64, _f64p, _f64p, _f64p, _vp, _INT, _vp, _INT, _I64,
        _f64p,
    ]
    L.fo_edge_topology.restype = _INT
    L.fo_edge_topology.argtypes = [
        _i64p, _I64, _INT, _i64p, _i64p, _i8p, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
    ]
    L.fo_integrate_tet_n1.restype = _INT
    L.fo_integrate_tet_n1.argtypes = [
        _f64p, _f64p, _f64p, _f64p, _f64p, _I64, _I64, _INT, _INT, _INT, _f64p,
    ]
    L.fo_add_at.argtypes = [_f64p, _I64, _i64p, _f64p, _I64]
    _lib = L
    return L


def max_threads() -> int:
    return int(lib().fo_max_threads())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


# --------------------------------------------------------------------------
# Meshes: python/skfemntv/basis.py:599-616 (MeshTet.init_tensor) and
# 644-658 (MeshTet2.from_mesh: first-seen edge nodes at midpoints).

HEX_TO_TETS = ((0, 1, 3, 7), (0, 3, 2, 7), (0, 2, 6, 7), (0, 6, 4, 7), (0, 4, 5, 7), (0, 5, 1, 7))
TET_EDGES = ((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3))


def mesh_tet_tensor(x, y, z):
    """Vertex order i + nx*(j + ny*k); cubes k -> j -> i; six tets per cube."""
    x, y, z = (np.asarray(a, dtype=np.float64) for a in (x, y, z))
    nx, ny, nz = len(x), len(y), len(z)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    p = np.stack((X.ravel(), Y.ravel(), Z.ravel()))
    k, j, i = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()

    def node(a, b, c):
        return a + nx * (b + ny * c)

    cube = np.stack([
        node(i, j, k), node(i + 1, j, k), node(i, j + 1, k), node(i + 1, j + 1, k),
        node(i, j, k + 1), node(i + 1, j, k + 1), node(i, j + 1, k + 1), node(i + 1, j + 1, k + 1),
    ])  # (8, ncubes)
    tets = np.stack([cube[list(pat)] for pat in HEX_TO_TETS], axis=1)  # (4, 6, ncubes)
    t = tets.transpose(0, 2, 1).reshape(4, -1)  # cube-major, then pattern
    return p, t.astype(np.int64)


def edge_topology(t4):
    """edge_topology.cpp:30-84 -> (edges (2,nE), element_edges (6,E), signs (6,E))."""
    t4 = np.ascontiguousarray(t4, dtype=np.int64)
    ne = t4.shape[1]
    edges = np.empty((2, max(1, 6 * ne)), dtype=np.int64)
    ee = np.empty((6, ne), dtype=np.int64)
    sg = np.empty((6, ne), dtype=np.int8)
    n = _I64(0)
    bad = _I64(-1)
    rc = lib().fo_edge_topology(t4, ne, 3, edges, ee, sg, ctypes.byref(n), ctypes.byref(bad))
    if rc != 0:
        raise ValueError(f"cell {bad.value} repeats a corner vertex")
    return np.ascontiguousarray(edges[:, : n.value]), ee, sg


def mesh_tet2_from_mesh(p, t):
    """P2 mesh: vertices then first-seen edge midpoints; t = 4 corners + 6 edges."""
    edges, ee, _ = edge_topology(t[:4])
    nv = p.shape[1]
    mid = 0.5 * (p[:, edges[0]] + p[:, edges[1]])
    return np.concatenate((p, mid), axis=1), np.vstack((t[:4], ee + nv)).astype(np.int64)


# --------------------------------------------------------------------------
# Quadrature: basis.py:1716-1734 (tet defaults), 1547-1561 (custom rule),
# hcurl_basis.py:37-56 (Duffy product rule).

def tet_quadrature_p1():
    a, b = 0.5854101966249685, 0.1381966011250105
    X = np.array([[a, b, b, b], [b, a, b, b], [b, b, a, b]])
    return X, np.full(4, 1.0 / 24.0)


def tet_quadrature_p2():
    X = np.array(
        [[.25, .7857142857142857, .0714285714285714, .0714285714285714, .0714285714285714,
          .1005964238332008, .3994035761667992, .3994035761667992, .3994035761667992,
          .1005964238332008, .1005964238332008],
         [.25, .0714285714285714, .0714285714285714, .0714285714285714, .7857142857142857,
          .3994035761667992, .1005964238332008, .3994035761667992, .1005964238332008,
          .3994035761667992, .1005964238332008],
         [.25, .0714285714285714, .0714285714285714, .7857142857142857, .0714285714285714,
          .3994035761667992, .3994035761667992, .1005964238332008, .1005964238332008,
          .1005964238332008, .3994035761667992]])
    W = np.array([-.01315555555555555] + [.00762222222222222] * 4 + [.02488888888888888] * 6)
    return X, W


def duffy_quadrature(order):
    count = max(1, (int(order) + 4) // 2)
    pts, wts = np.polynomial.legendre.leggauss(count)
    pts = (pts + 1.0) / 2.0
    wts = wts / 2.0
    X, W = [], []
    for f in range(count):
        for s in range(count):
            for r in range(count):
                x = pts[f]
                y = (1.0 - x) * pts[s]
                z = (1.0 - x) * (1.0 - pts[s]) * pts[r]
                X.append((x, y, z))
                W.append((1.0 - x) ** 2 * (1.0 - pts[s]) * wts[f] * wts[s] * wts[r])
    return np.asarray(X).T, np.asarray(W)


# --------------------------------------------------------------------------
# Reference tabulation: basis.py:2224-2240.

_DL = np.array([[-1., -1., -1.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.]])


def tabulate_reference(X, quadratic):
    nq = X.shape[1]
    if not quadratic:
        shape = np.vstack((1.0 - X.sum(axis=0), X)).T
        return np.ascontiguousarray(shape), np.ascontiguousarray(np.broadcast_to(_DL, (nq, 4, 3)))
    bary = np.vstack((1.0 - X.sum(axis=0), X)).T
    shape = np.empty((nq, 10))
    refgrad = np.empty((nq, 10, 3))
    for q, L in enumerate(bary):
        for i in range(4):
            shape[q, i] = L[i] * (2.0 * L[i] - 1.0)
            refgrad[q, i] = (4.0 * L[i] - 1.0) * _DL[i]
        for k, (i, j) in enumerate(TET_EDGES, start=4):
            shape[q, k] = 4.0 * L[i] * L[j]
            refgrad[q, k] = 4.0 * (L[j] * _DL[i] + L[i] * _DL[j])
    return shape, refgrad


# --------------------------------------------------------------------------
# Basis (nodal H1 over tets): DOF numbering basis.py:1749-1777; geometry
# basis.py:2194-2294 -> basis_geometry.cpp.

@dataclass
class OracleBasis:
    p: np.ndarray
    t: np.ndarray
    nodes: int
    comp: int
    X: np.ndarray
    W: np.ndarray
    N: int
    element_dofs: np.ndarray  # (nodes*comp, E)
    shape: np.ndarray         # (E, Q, nodes)
    grad: np.ndarray          # (E, Q, nodes, 3)
    dx: np.ndarray            # (E, Q)
    x: np.ndarray             # (E, Q, 3)
    det: np.ndarray
    tol: np.ndarray
    cond: np.ndarray

    @property
    def dofs3(self):
        E = self.t.shape[1]
        return np.ascontiguousarray(self.element_dofs.T.reshape(E, self.nodes, self.comp))


class GeometryError(ValueError):
    pass


def tabulate_geometry(p, t, X, W, quadratic, threads=1):
    """basis_geometry.cpp:49-209.  Geometry nodes are all rows of ``t``
    (isoparametric); a P1 element on a 10-node mesh uses the P2 geometry map
    (basis.py:2274-2283)."""
    p = np.ascontiguousarray(p, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.int64)
    G, E = t.shape
    shape, refgrad = tabulate_reference(X, quadratic)
    nq, n = shape.shape
    if G != n:
        if G < n:
            raise ValueError("mesh geometry nodes are incompatible with the element")
        gshape, gref = tabulate_reference(X, True)
    else:
        gshape, gref = shape, refgrad
    o_shape = np.zeros((E, nq, n)); o_grad = np.zeros((E, nq, n, 3)); o_dx = np.zeros((E, nq))
    o_x = np.zeros((E, nq, 3)); o_det = np.zeros((E, nq)); o_tol = np.zeros((E, nq))
    o_cond = np.zeros((E, nq))
    bc, bq, br = _I64(-1), _I64(-1), _INT(0)
    rc = lib().fo_tabulate_geometry(
        3, p.shape[1], p, G, E, t, nq, n, np.ascontiguousarray(shape), np.ascontiguousarray(refgrad),
        np.ascontiguousarray(gshape), np.ascontiguousarray(gref), np.ascontiguousarray(W),
        o_shape, o_grad, o_dx, o_x, o_det, o_tol, o_cond, threads,
        ctypes.byref(bc), ctypes.byref(bq), ctypes.byref(br),
    )
    if rc != 0:
        if br.value == 3:
            raise ValueError("connectivity index is out of bounds")
        e, q = bc.value, bq.value
        reason = "near_singular_or_non_finite" if br.value == 1 else "orientation_change"
        raise GeometryError(
            f"invalid element geometry: cell={e}, quadrature_point={q}, "
            f"determinant={o_det[e, q]:.17e}, tolerance={o_tol[e, q]:.17e}, reason={reason}"
        )
    return o_shape, o_grad, o_dx, o_x, o_det, o_tol, o_cond


def make_basis(p, t, quadratic, comp=1, quadrature=None, threads=1):
    nodes = 10 if quadratic else 4
    conn = t[:nodes]
    if quadrature is None:
        X, W = tet_quadrature_p2() if quadratic else tet_quadrature_p1()
    else:
        X, W = (np.ascontiguousarray(np.asarray(a, dtype=np.float64)) for a in quadrature)
    used = np.zeros(p.shape[1], dtype=bool)
    used[conn] = True
    active = np.flatnonzero(used)
    N = len(active) * comp
    nodal_dofs = np.arange(N).reshape(-1, comp).T
    pos = np.full(p.shape[1], -1, dtype=np.int64)
    pos[active] = np.arange(len(active))
    local = pos[conn]
    E = t.shape[1]
    element_dofs = nodal_dofs[:, local].transpose(2, 1, 0).reshape(E, nodes * comp).T
    o = tabulate_geometry(p, t, X, W, quadratic, threads=threads)
    return OracleBasis(p, t, nodes, comp, X, W, N, np.ascontiguousarray(element_dofs), *o)


# --------------------------------------------------------------------------
# Assembly drivers.

class Pattern:
    """fo_pattern handle (CSR pattern + scatter + coloring)."""

    def __init__(self, row_dofs, col_dofs=None, nrows=-1, coloring=True):
        row_dofs = np.ascontiguousarray(row_dofs, dtype=np.int64)
        col_dofs = row_dofs if col_dofs is None else np.ascontiguousarray(col_dofs, dtype=np.int64)
        self.ne = row_dofs.shape[0]
        self.h = lib().fo_pattern_build(
            row_dofs.reshape(self.ne, -1), col_dofs.reshape(self.ne, -1), self.ne,
            row_dofs.reshape(self.ne, -1).shape[1], col_dofs.reshape(self.ne, -1).shape[1],
            nrows, 1 if coloring else 0,
        )
        if not self.h:
            raise MemoryError("oracle pattern build failed")
        self.nnz = int(lib().fo_pattern_nnz(self.h))
        self.nrows = int(lib().fo_pattern_nrows(self.h))
        self.ncolors = int(lib().fo_pattern_ncolors(self.h))
        self.lr = row_dofs.reshape(self.ne, -1).shape[1]
        self.lc = col_dofs.reshape(self.ne, -1).shape[1]

    def csr(self, with_scatter=False):
        indptr = np.empty(self.nrows + 1, dtype=np.int64)
        indices = np.empty(self.nnz, dtype=np.int64)
        sc = np.empty((self.ne, self.lr, self.lc), dtype=np.int64) if with_scatter else None
        lib().fo_pattern_copy(self.h, _ptr(indptr), _ptr(indices), _ptr(sc))
        return (indptr, indices, sc) if with_scatter else (indptr, indices)

    def __del__(self):
        if getattr(self, "h", None):
            lib().fo_pattern_free(self.h)
            self.h = None


def _qcoef(c, shape):
    if c is None:
        return None
    return np.ascontiguousarray(np.broadcast_to(np.asarray(c, dtype=np.float64), shape))


def bilinear_assemble(basis: OracleBasis, value=None, gradient=None, symmetric_gradient=None,
                      divergence=None, threads=1, pattern=None):
    """NativeBilinearForm.assemble -> BilinearFormAssembler (values, indptr, indices)."""
    pat = pattern or Pattern(basis.dofs3.reshape(basis.dofs3.shape[0], -1))
    shp = basis.dx.shape
    v, g, s, d = (_qcoef(c, shp) for c in (value, gradient, symmetric_gradient, divergence))
    out = np.empty(pat.nnz)
    rc = lib().fo_bilinear_assemble(
        pat.h, basis.nodes, basis.comp, shp[1], 3, np.ascontiguousarray(basis.shape),
        np.ascontiguousarray(basis.grad), np.ascontiguousarray(basis.dx),
        _ptr(v), _ptr(g), _ptr(s), _ptr(d), threads, out,
    )
    if rc != 0:
        raise ValueError("at least one coefficient is required")
    indptr, indices = pat.csr()
    return out, indptr, indices


def anisotropic_tensor(raw, coefficient_shape, dim=3):
    """forms.py:377-404: (3,3) / (3,3,E,Q) / (E,Q,3,3) -> (E,Q,1,3,1,3)."""
    tensor = np.asarray(raw, dtype=np.float64)
    if tensor.shape == (dim, dim):
        tensor = np.broadcast_to(tensor, coefficient_shape + (dim, dim))
    elif tensor.shape == (dim, dim) + coefficient_shape:
        tensor = np.moveaxis(tensor, (0, 1), (-2, -1))
    elif tensor.shape == coefficient_shape + (dim, dim):
        pass
    else:
        raise ValueError("anisotropic tensor has an invalid shape")
    return np.ascontiguousarray(tensor[..., None, :, None, :])


def cross_gradient_tensor_assemble(basis: OracleBasis, tensor6, threads=1, pattern=None):
    """CrossBilinearAssembler.assemble(tensor, 'gradient', 'gradient') for one basis."""
    dofs = basis.dofs3.reshape(basis.dofs3.shape[0], -1)
    pat = pattern or Pattern(dofs, dofs)
    E, Q = basis.dx.shape
    C = basis.comp
    tensor6 = np.ascontiguousarray(np.broadcast_to(tensor6, (E, Q, C, 3, C, 3)), dtype=np.float64)
    out = np.empty(pat.nnz)
    sh = np.ascontiguousarray(basis.shape)
    gr = np.ascontiguousarray(basis.grad)
    rc = lib().fo_cross_assemble(
        pat.h, basis.nodes, basis.nodes, C, C, Q, 3, 3, sh, sh, _ptr(gr), _ptr(gr),
        np.ascontiguousarray(basis.dx), _ptr(tensor6), 1, 1, 1, threads, out,
    )
    if rc != 0:
        raise ValueError("cross assembly failed")
    indptr, indices = pat.csr()
    return out, indptr, indices


def linear_assemble(basis: OracleBasis, value=None, gradient=None):
    """NativeLinearForm.assemble (serial path): value (E,Q,C)|(C,), gradient (E,Q,C,3)|(C,3)."""
    E, Q = basis.dx.shape
    C = basis.comp
    vc = gc = 0
    if value is not None:
        value = np.asarray(value, dtype=np.float64)
        vc = int(value.shape == (C,))
        value = np.ascontiguousarray(value if vc else np.broadcast_to(value, (E, Q, C)))
    if gradient is not None:
        gradient = np.asarray(gradient, dtype=np.float64)
        gc = int(gradient.shape == (C, 3))
        gradient = np.ascontiguousarray(gradient if gc else np.broadcast_to(gradient, (E, Q, C, 3)))
    out = np.empty(basis.N)
    rc = lib().fo_linear_assemble(
        basis.dofs3.reshape(-1).copy(), E, basis.nodes, C, Q, 3, np.ascontiguousarray(basis.shape),
        np.ascontiguousarray(basis.grad), np.ascontiguousarray(basis.dx), _ptr(value), vc,
        _ptr(gradient), gc, basis.N, out,
    )
    if rc != 0:
        raise ValueError("at least one coefficient is required")
    return out


# --------------------------------------------------------------------------
# Nedelec N1 on tets: hcurl_basis.py:292-364, _hcurl_mapping.py:21-97,
# _nedelec_reference.py:72-107, hcurl_assembler.py:52-215.

_TET_BGRAD = _DL


def tet_n1_reference(X):
    lam = np.concatenate(((1.0 - X.sum(axis=0))[None], X), axis=0)
    vals = np.empty((6, 3) + X.shape[1:])
    for k, (a, b) in enumerate(TET_EDGES):
        vals[k] = lam[a][None] * _TET_BGRAD[b][:, None] - lam[b][None] * _TET_BGRAD[a][:, None]
    curls = np.array([2.0 * np.cross(_TET_BGRAD[a], _TET_BGRAD[b]) for a, b in TET_EDGES])
    return vals, np.broadcast_to(curls[:, :, None], (6, 3) + X.shape[1:]).copy()


@dataclass
class OracleN1Basis:
    N: int
    element_dofs: np.ndarray  # (6, E)
    signs: np.ndarray         # (6, E)
    edges: np.ndarray
    X: np.ndarray
    W: np.ndarray
    detJ: np.ndarray
    dx: np.ndarray            # (E, Q)
    values: np.ndarray        # (E, 6, 3, Q)
    curls: np.ndarray         # (E, 6, 3, Q)


def make_n1_basis(p, t, intorder=2):
    edges, ee, sg = edge_topology(t[:4])
    X, W = duffy_quadrature(intorder)
    v = p[:, t[:4]]
    J = np.stack(tuple(v[:, k] - v[:, 0] for k in (1, 2, 3)), axis=1)  # (3,3,E)
    det = (J[0, 0] * (J[1, 1] * J[2, 2] - J[1, 2] * J[2, 1])
           - J[0, 1] * (J[1, 0] * J[2, 2] - J[1, 2] * J[2, 0])
           + J[0, 2] * (J[1, 0] * J[2, 1] - J[1, 1] * J[2, 0]))
    if np.any(np.isclose(det, 0.0)):
        raise ValueError("H(curl) basis requires nonsingular tetrahedra")
    dx = np.abs(det)[:, None] * W[None, :]
    ref_v, ref_c = tet_n1_reference(X)
    inv = np.linalg.inv(np.moveaxis(J[..., None], (0, 1), (-2, -1)))
    inv = np.moveaxis(inv, (-2, -1), (0, 1))
    vals = np.einsum("rp...,br...->bp...", inv, ref_v[:, :, None, :]).transpose(2, 0, 1, 3)
    curls = (np.einsum("pr...,br...->bp...", J[..., None], ref_c[:, :, None, :]) / det[:, None]).transpose(2, 0, 1, 3)
    vals = np.ascontiguousarray(vals * sg.T[:, :, None, None])
    curls = np.ascontiguousarray(curls * sg.T[:, :, None, None])
    return OracleN1Basis(edges.shape[1], ee, sg, edges, X, W, det, dx, vals, curls)


def n1_assemble_maxwell(b: OracleN1Basis, mass_coefficient=None, curl_coefficient=None,
                        threads=1, pattern=None):
    E, Q = b.dx.shape
    mass = np.ascontiguousarray(np.broadcast_to(
        np.asarray(1.0 if mass_coefficient is None else mass_coefficient, dtype=np.float64), (E, Q)))
    curl = np.ascontiguousarray(np.broadcast_to(
        np.asarray(1.0 if curl_coefficient is None else curl_coefficient, dtype=np.float64), (E, Q)))
    pat = pattern or Pattern(np.ascontiguousarray(b.element_dofs.T), nrows=b.N, coloring=False)
    indptr, indices, scatter = pat.csr(with_scatter=True)
    el = np.empty((E, 6, 6))
    lib().fo_integrate_tet_n1(b.values, b.curls, np.ascontiguousarray(b.dx), mass, curl, E, Q,
                              1, 1, threads, el)
    data = np.empty(pat.nnz)
    lib().fo_add_at(data, pat.nnz, np.ascontiguousarray(scatter.ravel()), el.ravel(), el.size)
    return data, indptr, indices


def n1_element_matrices(b: OracleN1Basis, mass_coefficient=None, curl_coefficient=None, include_mass=True,
                        include_curl=True):
    """integrate_tet_n1 (edge_topology.cpp:156-233), the (E, 6, 6) element
    matrices; with one term included these are
    AffineTetN1Basis.element_mass_matrices / element_curl_curl_matrices
    (hcurl_basis.py:376-386)."""
    E, Q = b.dx.shape
    mass = np.ascontiguousarray(np.broadcast_to(
        np.asarray(1.0 if mass_coefficient is None else mass_coefficient, dtype=np.float64), (E, Q)))
    curl = np.ascontiguousarray(np.broadcast_to(
        np.asarray(1.0 if curl_coefficient is None else curl_coefficient, dtype=np.float64), (E, Q)))
    el = np.empty((E, 6, 6))
    lib().fo_integrate_tet_n1(b.values, b.curls, np.ascontiguousarray(b.dx), mass, curl, E, Q,
                              int(include_mass), int(include_curl), 1, el)
    return el


def n1_evaluate(b: OracleN1Basis, coefficients, curl=False):
    """AffineTetN1Basis.evaluate / evaluate_curl (hcurl_basis.py:418-432):
    the global edge field at the rule's points, (3, E, Q)."""
    local = np.asarray(coefficients, dtype=np.float64)[b.element_dofs].T
    return np.einsum("eb,ebiq->ieq", local, b.curls if curl else b.values)


def n1_interpolate_edge_moments(p, edges, field, quadrature_order=4):
    """AffineTetN1Basis.interpolate_edge_moments (hcurl_basis.py:388-416):
    Gauss-Legendre tangential moments along each ascending global edge, the
    field called once per edge."""
    nodes, weights = np.polynomial.legendre.leggauss(int(quadrature_order))
    param = 0.5 * (nodes + 1.0)
    weights = 0.5 * weights
    out = np.empty(edges.shape[1])
    for k, (a, b) in enumerate(edges.T):
        first = p[:, a]
        tangent = p[:, b] - first
        pts = first[:, None] + tangent[:, None] * param[None, :]
        vals = np.broadcast_to(np.asarray(field(pts), dtype=np.float64), pts.shape)
        out[k] = np.einsum("iq,i,q->", vals, tangent, weights)
    return out


def n1_vector_load(b: OracleN1Basis, f):
    """TetN1LinearAssembler.assemble_vector_load (hcurl_assembler.py:218-246):
    local_eb = sum_iq phi_ebiq f_ieq dx_eq, summed into the edge DOFs in
    (element, local edge) order."""
    f = np.broadcast_to(np.asarray(f, dtype=np.float64), (3,) + b.dx.shape)
    local = np.einsum("ebiq,ieq,eq->eb", b.values, f, b.dx)
    out = np.zeros(b.N)
    np.add.at(out, b.element_dofs.T.ravel(), local.ravel())
    return out


def n1_global_coordinates(p, t, X):
    """Physical quadrature points (3, E, Q) of the affine map (hcurl_basis.py:435-440)."""
    v = p[:, t[:4]]
    J = np.stack([v[:, k] - v[:, 0] for k in (1, 2, 3)], axis=1)  # (3, 3, E): [i, r, e]
    return v[:, 0][:, :, None] + np.einsum("ire,rq->ieq", J, X)


# --------------------------------------------------------------------------
# Neo-Hookean law: benchmarks/skfem_neo_hookean.py:8-52 (residual P and the
# tangent tensor), with W = mu/2 (I1-3) - mu ln J + lambda/2 (ln J)^2.

def displacement_gradient(basis: OracleBasis, u):
    """grad u at quadrature points, (E,Q,3,3) with [c, j] = d u_c / d x_j."""
    ul = np.asarray(u)[basis.dofs3]  # (E, nodes, comp)
    return np.einsum("eac,eqaj->eqcj", ul, basis.grad)


def nh_first_piola(Gu, mu, lmbda):
    F = np.eye(3) + Gu
    FiT = np.swapaxes(np.linalg.inv(F), -1, -2)
    lnJ = np.log(np.linalg.det(F))
    return mu * (F - FiT) + lmbda * lnJ[..., None, None] * FiT


def nh_tangent(Gu, mu, lmbda):
    """A[..., r, i, c, j]: test (r,i) x trial (c,j), the cross-assembler layout."""
    F = np.eye(3) + Gu
    FiT = np.swapaxes(np.linalg.inv(F), -1, -2)
    lnJ = np.log(np.linalg.det(F))
    I = np.eye(3)
    A = mu * np.einsum("rc,ij->ricj", I, I) * np.ones(lnJ.shape)[..., None, None, None, None]
    A = A + (mu - lmbda * lnJ)[..., None, None, None, None] * np.einsum("...rj,...ci->...ricj", FiT, FiT)
    A = A + lmbda * np.einsum("...ri,...cj->...ricj", FiT, FiT)
    return A


def nh_energy(F, mu, lmbda):
    J = np.linalg.det(F)
    I1 = np.einsum("...ij,...ij->...", F, F)
    lnJ = np.log(J)
    return 0.5 * mu * (I1 - 3.0) - mu * lnJ + 0.5 * lmbda * lnJ ** 2


# --------------------------------------------------------------------------
# Energy surrogate network (no counterpart in the reference): FP64 numpy
# restatement of the MLP 3 -> 64 -> 64 -> 1 (tanh) with a linear skip
# (psi = w3 . z2 + b3 + c . x) and of its training loss, the checker for the
# GPU network kernels.  Parameter layout: W1 (64,3), b1, W2 (64,64), b2,
# w3 (64), b3, c (3), then f_mean (3), f_std (3), y_scale, y_shift, stress
# shift.

MLP_H = 64


def mlp_unpack(params):
    p = np.asarray(params, dtype=np.float64)
    H = MLP_H
    o = 0
    W1 = p[o:o + 3 * H].reshape(H, 3); o += 3 * H
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]; o += 1
    c = p[o:o + 3]; o += 3
    norm = p[o:o + 9]
    return W1, b1, W2, b2, w3, b3, c, norm


MLP_N_TRAINABLE = 3 * MLP_H + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1 + 3


def mlp_eval(params, x):
    """psi, grad psi (n,3), Hessian (n,3,3) at normalised inputs x (n,3)."""
    W1, b1, W2, b2, w3, b3, c, _ = mlp_unpack(params)
    x = np.asarray(x, dtype=np.float64)
    z1 = np.tanh(x @ W1.T + b1)
    s1 = 1 - z1 ** 2
    z2 = np.tanh(z1 @ W2.T + b2)
    s2 = 1 - z2 ** 2
    psi = z2 @ w3 + b3 + x @ c
    d2 = s2 * w3
    u1 = d2 @ W2
    d1 = s1 * u1
    g = d1 @ W1 + c
    Hm = np.empty((x.shape[0], 3, 3))
    for m in range(3):
        da1 = W1[:, m][None, :]
        dz1 = s1 * da1
        da2 = dz1 @ W2.T
        dd2 = -2 * z2 * s2 * da2 * w3
        du1 = dd2 @ W2
        dd1 = -2 * z1 * s1 * da1 * u1 + s1 * du1
        Hm[:, :, m] = dd1 @ W1
    return psi, g, Hm


def mlp_loss(params, feats, tgts, beta=1.0):
    """Mean of (psi - t)^2 + beta |grad psi - t'|^2 in normalised units."""
    norm = mlp_unpack(params)[-1]
    fm, fs, ys, yc = norm[:3], norm[3:6], norm[6], norm[7]
    x = (np.asarray(feats, np.float64) - fm) / fs
    t = (np.asarray(tgts[:, 0], np.float64) - yc) / ys
    tg = np.asarray(tgts[:, 1:], np.float64) * fs / ys
    psi, g, _ = mlp_eval(params, x)
    return float(np.mean((psi - t) ** 2 + beta * np.sum((g - tg) ** 2, axis=1)))
