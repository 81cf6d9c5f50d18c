"""Form front end on the GPU with the reference's compatible-forms cases (tests/test_compatible_forms.py,
volume forms on a vector P1 basis with the default rule) against the oracle: constant and coordinate
dependent loads, a gradient load through ``LinearForm.assemble``, mass and elasticity forms, coordinate
and parameter dependent coefficients, several terms with subtraction, and the error for a foreign form."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
sk = pytest.importorskip("skfemntv_gb300")
from skfemntv_gb300.forms import ddot, div, dot, grad, sym_grad  # noqa: E402

RTOL = 1e-12


def relerr(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def bases():
    m = sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, 3),) * 3)
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=3), intorder=2)
    ob = O.make_basis(m.p, m.t, False, comp=3, quadrature=(b.X, b.W))
    return b, ob


def test_linear_forms(bases):
    b, ob = bases

    @sk.LinearForm
    def load(v, w):
        return dot(w.force, v)

    force = np.array([1.2, -0.7, 2.1])
    assert relerr(sk.asm(load, b, force=force[:, None, None]), O.linear_assemble(ob, value=force)) < RTOL

    @sk.LinearForm
    def gradient_load(v, w):
        return ddot(w.tensor, grad(v))

    tensor = np.arange(9, dtype=float).reshape(3, 3) / 10
    got = gradient_load.assemble(b, tensor=tensor[:, :, None, None])
    assert relerr(got, O.linear_assemble(ob, gradient=tensor)) < RTOL

    def field(x):
        return np.stack((1.0 + x[0], x[1] ** 2, -0.5 * x[2]), axis=0)

    @sk.LinearForm
    def coordinate_load(v, w):
        return dot(field(w.x), v)

    x = np.moveaxis(b.global_coordinates, -1, 0)
    want = O.linear_assemble(ob, value=np.moveaxis(field(x), 0, -1))
    assert relerr(sk.asm(coordinate_load, b), want) < RTOL


def test_bilinear_forms(bases):
    b, ob = bases
    x = np.moveaxis(b.global_coordinates, -1, 0)

    @sk.BilinearForm
    def mass(u, v, w):
        return dot(u, v)

    K = sk.asm(mass, b)
    d, indptr, indices = O.bilinear_assemble(ob, value=1.0)
    assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
    assert relerr(K.data, d) < RTOL

    lam, mu = 2.3, 0.7

    @sk.BilinearForm
    def elasticity(u, v, w):
        return 2.0 * mu * ddot(sym_grad(u), sym_grad(v)) + lam * div(u) * div(v)

    assert relerr(sk.asm(elasticity, b).data,
                  O.bilinear_assemble(ob, symmetric_gradient=2.0 * mu, divergence=lam)[0]) < RTOL

    @sk.BilinearForm
    def weighted_mass(u, v, w):
        return (1.0 + w.x[0] ** 2) * dot(u, v)

    assert relerr(sk.asm(weighted_mass, b).data, O.bilinear_assemble(ob, value=1.0 + x[0] ** 2)[0]) < RTOL

    @sk.BilinearForm
    def scaled_mass(u, v, w):
        return w.scale * (1.0 + w.x[0]) * dot(u, v)

    assert relerr(sk.asm(scaled_mass, b, scale=1.8).data,
                  O.bilinear_assemble(ob, value=1.8 * (1.0 + x[0]))[0]) < RTOL

    @sk.BilinearForm
    def reaction_diffusion(u, v, w):
        return (w.reaction * (1.0 + w.x[0] ** 2) * dot(u, v)
                + w.diffusivity * np.exp(-w.x[1]) * ddot(grad(u), grad(v)))

    got = sk.asm(reaction_diffusion, b, reaction=1.3, diffusivity=0.4).data
    want = O.bilinear_assemble(ob, value=1.3 * (1.0 + x[0] ** 2), gradient=0.4 * np.exp(-x[1]))[0]
    assert relerr(got, want) < RTOL

    @sk.BilinearForm
    def with_subtraction(u, v, w):
        return 2.0 * dot(u, v) + 3.0 * ddot(grad(u), grad(v)) - 0.5 * dot(u, v) - ddot(grad(u), grad(v))

    @sk.BilinearForm
    def reduced(u, v, w):
        return 1.5 * dot(u, v) + 2.0 * ddot(grad(u), grad(v))

    np.testing.assert_allclose(sk.asm(with_subtraction, b).toarray(), sk.asm(reduced, b).toarray())

    def foreign(v, w):
        return v[0]

    with pytest.raises(TypeError, match="use skfem.asm explicitly"):
        sk.asm(foreign, b)
