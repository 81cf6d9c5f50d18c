"""Tetrahedral meshes (python/skfemntv/basis.py:581-669).

``MeshTet.init_tensor`` builds the same vertex numbering (i + nx (j + ny k))
and the same six-tetrahedra split of every hexahedron, in the same cube order
(k, j, i), as the reference; it is vectorised.  ``MeshTet2.from_mesh`` adds
the edge midpoints numbered in first-seen order, computed on the GPU by the
oriented-edge kernel (the reference walks a Python dict, basis.py:644-658).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _device as dev
from ._native import call

_HEX_TETS = ((0, 1, 3, 7), (0, 3, 2, 7), (0, 2, 6, 7), (0, 6, 4, 7), (0, 4, 5, 7), (0, 5, 1, 7))


class MeshTet:
    """Linear tetrahedral mesh: p (3, npts) float64, t (4, nelements) int64."""

    def __init__(self, p=None, t=None):
        self.p = np.asarray(
            p if p is not None else [[0., 1., 0., 0.], [0., 0., 1., 0.], [0., 0., 0., 1.]],
            dtype=np.float64)
        self.t = np.asarray(t if t is not None else [[0], [1], [2], [3]], dtype=np.int64)
        if self.p.ndim != 2 or self.p.shape[0] != 3:
            raise ValueError("p must have shape (3, nodes)")
        if self.t.ndim != 2 or self.t.shape[0] != 4:
            raise ValueError("t must have shape (4, elements)")
        self._device_cache = {}

    @classmethod
    def init_tensor(cls, x, y, z):
        x, y, z = (np.asarray(a, dtype=np.float64) for a in (x, y, z))
        nx, ny, nz = len(x), len(y), len(z)
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        p = np.stack((X.ravel(), Y.ravel(), Z.ravel()))
        k, j, i = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
        i, j, k = i.ravel(), j.ravel(), k.ravel()
        n0 = i + nx * (j + ny * k)
        dx, dy, dz = 1, nx, nx * ny
        cube = np.stack([n0, n0 + dx, n0 + dy, n0 + dx + dy, n0 + dz, n0 + dx + dz, n0 + dy + dz,
                         n0 + dx + dy + dz])
        t = np.stack([cube[list(pat)] for pat in _HEX_TETS], axis=1)  # (4, 6, ncubes)
        return cls(p, t.transpose(0, 2, 1).reshape(4, -1).astype(np.int64))

    @property
    def nelements(self):
        return self.t.shape[1]

    def dim(self):
        return 3

    # device copies, created on first use and reused by every basis
    def _dev(self, name):
        cache = self.__dict__.setdefault("_device_cache", {})
        if name not in cache:
            if name == "p":
                cache[name] = dev.to_device(self.p, np.float64)
            elif name == "t":
                if self.t.size and (self.t.min() < 0 or self.t.max() >= self.p.shape[1]):
                    raise ValueError("connectivity index is out of bounds")
                cache[name] = dev.to_device(self.t, np.int32)
            else:
                raise KeyError(name)
        return cache[name]


def oriented_edges(t4_device, nelements):
    """First-seen global edges of a tetrahedral connectivity (device (4, E) int32).

    Returns (edges (2, nE) int64 host, element_edges (6, E) device int32,
    signs (6, E) device int8)."""
    edges = dev.empty((2, max(1, 6 * nelements)), np.int32)
    ee = dev.empty((6, nelements), np.int32)
    sg = dev.empty((6, nelements), np.int8)
    n = ctypes.c_int64(0)
    bad = ctypes.c_int64(-1)
    call("skg_edge_topology", dev.ptr(t4_device), nelements, dev.ptr(edges), dev.ptr(ee), dev.ptr(sg),
         ctypes.byref(n), ctypes.byref(bad), dev.stream_ptr())
    ne = n.value
    e_host = edges.cpu().numpy()
    return np.ascontiguousarray(e_host[:, :ne].astype(np.int64)), ee, sg


class MeshTet2(MeshTet):
    """Quadratic tetrahedral mesh: 4 vertices + 6 shared edge nodes per element."""

    @classmethod
    def from_mesh(cls, mesh: MeshTet):
        t4 = mesh._dev("t")[:4].contiguous()
        edges, ee, _ = oriented_edges(t4, mesh.nelements)
        nv = mesh.p.shape[1]
        mid = 0.5 * (mesh.p[:, edges[0]] + mesh.p[:, edges[1]])
        t = np.vstack((mesh.t[:4], ee.cpu().numpy().astype(np.int64) + nv))
        return cls(np.concatenate((mesh.p, mid), axis=1), t)

    def __init__(self, p=None, t=None):
        if p is None or t is None:
            # the reference tetrahedron with its six edge nodes in local order
            base = MeshTet()
            order = [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]
            mids = [0.5 * (base.p[:, min(a, b)] + base.p[:, max(a, b)]) for a, b in order]
            self.p = np.concatenate((base.p, np.stack(mids, axis=1)), axis=1)
            self.t = np.arange(10, dtype=np.int64)[:, None]
            self._device_cache = {}
            return
        self.p = np.asarray(p, dtype=np.float64)
        self.t = np.asarray(t, dtype=np.int64)
        if self.p.ndim != 2 or self.p.shape[0] != 3 or self.t.ndim != 2 or self.t.shape[0] != 10:
            raise ValueError("quadratic tetra mesh requires p (3,n) and t (10,e)")
        self._device_cache = {}
