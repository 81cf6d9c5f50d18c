"""Degenerate sizes on the GPU path, with the reference's behaviour (checked
by running the reference on the same inputs): a single element, vertices no
element uses (compacted out of the DOF numbering, basis.py:1764-1766) and an
empty mesh (an empty (0, 0) matrix)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
sk = pytest.importorskip("skfemntv_gb300")
from skfemntv_gb300.forms import ddot, dot, grad, mul  # noqa: E402

X1 = np.array([[.25], [.25], [.25]])
W1 = np.array([1 / 6])
P = np.array([[0., 1., 0., 0.], [0., 0., 1., 0.], [0., 0., 0., 1.]])
T = np.array([[0], [1], [2], [3]])


@sk.BilinearForm
def lap(u, v, w):
    return ddot(grad(u), grad(v))


@sk.BilinearForm
def aniso(u, v, w):
    return dot(mul(w.A, grad(u)), grad(v))


def relerr(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def p1(p, t):
    return sk.Basis(sk.MeshTet(p, t), sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X1, W1))


def test_single_element_p1_and_p2():
    K = sk.asm(lap, p1(P, T))
    ob = O.make_basis(P, T, False, quadrature=(X1, W1))
    data, indptr, indices = O.bilinear_assemble(ob, gradient=1.0)
    assert K.shape == (4, 4) and K.nnz == 16
    assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
    assert relerr(K.data, data) < 1e-12
    m2 = sk.MeshTet2.from_mesh(sk.MeshTet(P, T))
    X, W = O.tet_quadrature_p2()
    b2 = sk.Basis(m2, sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(X, W))
    A = np.array([[2.0, 0.3, 0.1], [0.3, 1.5, 0.2], [0.1, 0.2, 1.0]])
    E, Q = b2._coefficient_shape
    K2 = sk.asm(aniso, b2, A=np.broadcast_to(A[:, :, None, None], (3, 3, E, Q)))
    ob2 = O.make_basis(m2.p, m2.t, True, quadrature=(X, W))
    tensor = O.anisotropic_tensor(np.broadcast_to(A[:, :, None, None], (3, 3, E, Q)), (E, Q))
    d2, ip2, ix2 = O.cross_gradient_tensor_assemble(ob2, tensor)
    assert K2.shape == (10, 10) and np.array_equal(K2.indptr, ip2) and np.array_equal(K2.indices, ix2)
    assert relerr(K2.data, d2) < 1e-12


def test_unused_vertices_are_compacted():
    K = sk.asm(lap, p1(P, T)).copy()
    far = np.array([[5.0], [5.0], [5.0]])
    b_last = p1(np.hstack([P, far]), T)
    b_first = p1(np.hstack([far, P]), T + 1)
    assert b_last.N == 4 and b_first.N == 4
    for b in (b_last, b_first):
        Kb = sk.asm(lap, b)
        assert Kb.shape == (4, 4)
        assert np.array_equal(Kb.indptr, K.indptr) and np.array_equal(Kb.indices, K.indices)
        assert np.array_equal(Kb.data, K.data)


def test_empty_mesh_gives_empty_matrix():
    b = p1(P, np.zeros((4, 0), dtype=np.int64))
    assert b.N == 0
    K = sk.asm(lap, b)
    assert K.shape == (0, 0) and K.nnz == 0


def test_single_element_n1_maxwell():
    nb = sk.AffineTetN1Basis(sk.MeshTet(P, T))
    K = sk.TetN1Assembler(nb).assemble_maxwell(mass_coefficient=2.0, curl_coefficient=0.5)
    ob = O.make_n1_basis(P, T)
    data, indptr, indices = O.n1_assemble_maxwell(ob, 2.0, 0.5)
    assert K.shape == (6, 6) and K.nnz == 36
    assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
    assert relerr(K.data, data) < 1e-12


def test_fused_p1_forms_degenerate_meshes():
    """The fused affine P1 forms path (per-element coefficients) on a single element, with an unused vertex
    (compacted out of the DOF numbering) and as a P1 field on a P2 geometry mesh (affine: vertex rows only)."""
    from skfemntv_gb300.assembly import NativeBilinearForm

    kinds = dict(value=0.5, gradient=1.25, symmetric_gradient=2.0, divergence=10.0)
    for comp in (1, 3):
        # single element, and the same element with a far vertex no element uses (DOF numbering compacts it)
        for p, t in ((P, T), (np.concatenate([np.array([[5.0], [5.0], [5.0]]), P], axis=1), T + 1)):
            b = sk.Basis(sk.MeshTet(p, t), sk.ElementVector(sk.ElementTetP1(), dim=comp))
            K = NativeBilinearForm(b).assemble(**kinds)
            assert b._tab is None  # fused path
            ob = O.make_basis(p, t, False, comp=comp)
            data, indptr, indices = O.bilinear_assemble(ob, **kinds)
            assert K.shape == (4 * comp, 4 * comp)
            assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
            assert relerr(K.data, data) < 1e-12
        # P1 field on the quadratic geometry mesh of a jittered cube: the map is affine, vertex rows are used
        m = sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, 3),) * 3)
        m2 = sk.MeshTet2.from_mesh(m)
        b = sk.Basis(m2, sk.ElementVector(sk.ElementTetP1(), dim=comp))
        assert b.is_affine
        K = NativeBilinearForm(b).assemble(**kinds)
        ob = O.make_basis(m2.p, m2.t, False, comp=comp)
        data, indptr, indices = O.bilinear_assemble(ob, **kinds)
        assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
        assert relerr(K.data, data) < 1e-12
