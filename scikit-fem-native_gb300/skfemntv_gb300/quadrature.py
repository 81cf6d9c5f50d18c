"""Quadrature rules on the unit tetrahedron.

The default rules are the reference's (python/skfemntv/basis.py:1716-1734:
the symmetric 4-point rule for P1 and the 11-point Keast rule, with its
negative centroid weight, for P2), restated as data; the Duffy product rule
of the H(curl) basis (python/skfemntv/hcurl_basis.py:37-56) and the
collapsed Gauss-Legendre rule the H1 basis takes above order 4
(basis.py:1580-1598) are computed with the reference's arithmetic.  The
points and weights must be the same numbers for results to agree.
"""
from __future__ import annotations

import numpy as np

_A4, _B4 = 0.5854101966249685, 0.1381966011250105


def tet_rule_p1():
    X = np.array([[_A4, _B4, _B4, _B4], [_B4, _A4, _B4, _B4], [_B4, _B4, _A4, _B4]])
    return X, np.full(4, 1.0 / 24.0)


def tet_rule_p2():
    a, b, c, d = .25, .7857142857142857, .0714285714285714, .1005964238332008
    e = .3994035761667992
    X = np.array([
        [a, b, c, c, c, d, e, e, e, d, d],
        [a, c, c, c, b, e, d, e, d, e, d],
        [a, c, c, b, c, e, e, d, d, d, e],
    ])
    W = np.array([-.01315555555555555] + [.00762222222222222] * 4 + [.02488888888888888] * 6)
    return X, W


def duffy_rule(order):
    """Collapsed Gauss-Legendre product rule with count = (order+4)//2 per axis."""
    count = max(1, (int(order) + 4) // 2)
    g, gw = np.polynomial.legendre.leggauss(count)
    g = (g + 1.0) / 2.0
    gw = gw / 2.0
    X, W = [], []
    for i in range(count):
        for j in range(count):
            for k in range(count):
                x = g[i]
                y = (1.0 - x) * g[j]
                z = (1.0 - x) * (1.0 - g[j]) * g[k]
                X.append((x, y, z))
                W.append((1.0 - x) ** 2 * (1.0 - g[j]) * gw[i] * gw[j] * gw[k])
    return np.ascontiguousarray(np.asarray(X).T), np.asarray(W)


def simplex_rule(order):
    """The H1 basis's rule above order 4 on the unit tetrahedron
    (basis.py:1580-1598): Gauss-Legendre points t on [0, 1],
    (order + 4) // 2 per axis, collapsed as x = t0, y = (1 - t0) t1,
    z = ((1 - t0)(1 - t1)) t2 with weight (1 - t0)^2 (1 - t1) times
    (w0 w1) w2, the last axis fastest.  The products are grouped as there so
    that the rule is the same numbers (its weights group the 1-D weights
    differently from ``duffy_rule``)."""
    count = max(1, (int(order) + 4) // 2)
    g, gw = np.polynomial.legendre.leggauss(count)
    g = (g + 1.0) / 2.0
    gw = gw / 2.0
    i0, i1, i2 = (a.ravel() for a in np.indices((count, count, count)))
    rest = 1.0 - g
    # the square through the C library's pow, as a scalar power is taken there
    # (an array's ** 2 would multiply, which can round differently)
    rest_sq = np.array([float(r) ** 2 for r in rest])
    X = np.stack((g[i0], rest[i0] * g[i1], (rest[i0] * rest[i1]) * g[i2]))
    W = (rest_sq[i0] * rest[i1]) * ((gw[i0] * gw[i1]) * gw[i2])
    return np.ascontiguousarray(X), W


def validate(quadrature, dimension=3):
    """Custom (X, W): X (dim, nq), W (nq,), finite (basis.py:1547-1561)."""
    X, W = quadrature
    X = np.asarray(X, dtype=np.float64)
    W = np.asarray(W, dtype=np.float64)
    if X.ndim != 2 or X.shape[0] != dimension:
        raise ValueError(f"quadrature points must have shape ({dimension}, nq)")
    if W.ndim != 1 or W.shape[0] != X.shape[1]:
        raise ValueError("quadrature weights must have shape (nq,)")
    if not np.all(np.isfinite(X)) or not np.all(np.isfinite(W)):
        raise ValueError("quadrature points and weights must be finite")
    return np.ascontiguousarray(X), np.ascontiguousarray(W)


_DL = np.array([[-1., -1., -1.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.]])
TET_EDGES = ((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3))


def tabulate(X, quadratic):
    """Reference shapes (nq, n) and gradients (nq, n, 3) of P1/P2 at X
    (basis.py:2224-2240)."""
    nq = X.shape[1]
    lam = np.vstack((1.0 - X.sum(axis=0), X)).T  # (nq, 4)
    if not quadratic:
        return np.ascontiguousarray(lam), np.ascontiguousarray(np.broadcast_to(_DL, (nq, 4, 3)))
    shape = np.empty((nq, 10))
    grad = np.empty((nq, 10, 3))
    for i in range(4):
        shape[:, i] = lam[:, i] * (2.0 * lam[:, i] - 1.0)
        grad[:, i] = (4.0 * lam[:, i] - 1.0)[:, None] * _DL[i]
    for k, (i, j) in enumerate(TET_EDGES, start=4):
        shape[:, k] = 4.0 * lam[:, i] * lam[:, j]
        grad[:, k] = 4.0 * (lam[:, j][:, None] * _DL[i] + lam[:, i][:, None] * _DL[j])
    return shape, grad
