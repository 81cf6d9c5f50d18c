"""Form front end on the GPU with the reference's compatible-forms cases (tests/test_compatible_forms.py,
volume forms on a vector P1 basis with the default rule) against the reference's own outputs (fixture
forms_vp1): constant, gradient and coordinate-dependent loads, a gradient load through
``LinearForm.assemble``, mass and elasticity forms, coordinate and parameter dependent coefficients,
several terms with subtraction, and the error for a foreign form."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu
sk = pytest.importorskip("skfemntv_gb300")
from skfemntv_gb300.forms import ddot, div, dot, grad, sym_grad  # noqa: E402

RTOL = 1e-12


def relerr(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def case():
    g = load_golden("forms_vp1")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=3), intorder=2)
    assert np.array_equal(b.X, g["X"]) and np.array_equal(b.W, g["W"])
    return g, b


def test_linear_forms(case):
    g, b = case

    @sk.LinearForm
    def load(v, w):
        return dot(w.force, v)

    assert relerr(sk.asm(load, b, force=g["force"][:, None, None]), g["r_force"]) < RTOL
    # the assembler itself returns (vector, diagnostics) as the reference's (linear_form.py:62-89)
    r, diag = sk.NativeLinearForm(b).assemble(value=g["force"])
    assert relerr(r, g["r_force"]) < RTOL
    assert (diag.entity_count, diag.quadrature_point_count) == b.dx.shape and diag.assembly_seconds > 0

    @sk.LinearForm
    def gradient_load(v, w):
        return ddot(w.tensor, grad(v))

    assert relerr(gradient_load.assemble(b, tensor=g["tensor"]), g["r_tensor"]) < RTOL

    @sk.LinearForm
    def coordinate_load(v, w):
        x = w.x
        return dot(np.stack((1.0 + x[0], x[1] ** 2, -0.5 * x[2]), axis=0), v)

    assert relerr(sk.asm(coordinate_load, b), g["r_coordinate"]) < RTOL


def test_bilinear_forms(case):
    g, b = case

    @sk.BilinearForm
    def mass(u, v, w):
        return dot(u, v)

    K = sk.asm(mass, b)
    assert np.array_equal(K.indptr, g["indptr"]) and np.array_equal(K.indices, g["indices"])
    assert relerr(K.data, g["data"]) < RTOL

    @sk.BilinearForm
    def elasticity(u, v, w):
        return 2.0 * 0.7 * ddot(sym_grad(u), sym_grad(v)) + 2.3 * div(u) * div(v)

    assert relerr(sk.asm(elasticity, b).data, g["elasticity"]) < RTOL

    @sk.BilinearForm
    def weighted_mass(u, v, w):
        return (1.0 + w.x[0] ** 2) * dot(u, v)

    assert relerr(sk.asm(weighted_mass, b).data, g["weighted_mass"]) < RTOL

    @sk.BilinearForm
    def scaled_mass(u, v, w):
        return w.scale * (1.0 + w.x[0]) * dot(u, v)

    assert relerr(sk.asm(scaled_mass, b, scale=1.8).data, g["scaled_mass"]) < RTOL

    @sk.BilinearForm
    def reaction_diffusion(u, v, w):
        return (w.reaction * (1.0 + w.x[0] ** 2) * dot(u, v)
                + w.diffusivity * np.exp(-w.x[1]) * ddot(grad(u), grad(v)))

    got = sk.asm(reaction_diffusion, b, reaction=1.3, diffusivity=0.4).data
    assert relerr(got, g["reaction_diffusion"]) < RTOL

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
