"""Tetrahedral nodal elements (python/skfemntv/basis.py:933-937, 1006-1012,
1058-1061).  Local node order: the four vertices, then for P2 the six edge
midpoints of edges (0,1),(1,2),(2,0),(0,3),(1,3),(2,3)."""
from __future__ import annotations

import numpy as np


class ElementTetP1:
    def __init__(self):
        self.doflocs = np.array([[0., 0., 0.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.]])


class ElementTetP2:
    def __init__(self):
        self.doflocs = np.array(
            [[0., 0., 0.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.],
             [.5, 0., 0.], [.5, .5, 0.], [0., .5, 0.], [0., 0., .5],
             [.5, 0., .5], [0., .5, .5]])


class ElementVector:
    """`dim` copies of a scalar element; DOF = node position * dim + component."""

    def __init__(self, element, dim: int | None = None):
        self.elem = element
        self._dim = element.doflocs.shape[1] if dim is None else int(dim)
