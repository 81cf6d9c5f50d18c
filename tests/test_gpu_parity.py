"""GPU parity: the CUDA path through the public API / C ABI against the
reference's own outputs (tests/golden) and the CPU oracle.

Index structures (indptr, indices, edge ids, signs) must match exactly; FP64
values within 1e-12 relative to the largest entry (the tolerance the
reference's own FP64 contract states); geometry tabulation bit for bit.
"""
import numpy as np
import pytest

import oracle as O
from conftest import load_golden

pytestmark = pytest.mark.gpu

sk = pytest.importorskip("skfemntv_gb300")
from skfemntv_gb300.forms import ddot, dot, grad, mul, sym_grad, div  # noqa: E402

RTOL = 1e-12
X1 = np.array([[.25], [.25], [.25]])
W1 = np.array([1 / 6])


def relerr(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def same_pattern(K, g):
    assert np.array_equal(K.indptr, g["indptr"])
    assert np.array_equal(K.indices, g["indices"])


@sk.BilinearForm
def lap(u, v, w):
    return ddot(grad(u), grad(v))


@sk.BilinearForm
def lap_dot(u, v, w):
    return dot(grad(u), grad(v))


@sk.BilinearForm
def klap(u, v, w):
    return w.kappa * ddot(grad(u), grad(v))


@sk.BilinearForm
def aniso(u, v, w):
    return dot(mul(w.A, grad(u)), grad(v))


def test_p1_laplace_one_point():
    g = load_golden("p1_laplace")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X1, W1))
    K = sk.asm(lap, b)
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL
    K2 = sk.asm(lap_dot, b)
    assert relerr(K2.data, g["data"]) < RTOL
    Kk = sk.asm(klap, b, kappa=g["kappa"][:, None])
    assert relerr(Kk.data, g["kdata"]) < RTOL


def test_p1_reused_matrix_semantics():
    g = load_golden("p1_laplace")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X1, W1))
    K1 = sk.asm(klap, b, kappa=np.ones((b.mesh.nelements, 1)))
    d1 = K1.data.copy()
    K2 = sk.asm(klap, b, kappa=2 * np.ones((b.mesh.nelements, 1)))
    assert K1 is K2  # same object, values overwritten (bilinear_form.py:50-59)
    assert np.allclose(K2.data, 2 * d1, rtol=1e-15, atol=0)


def test_p1_mass_stiffness_tabulated_path():
    g = load_golden("p1_helmholtz")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=1))

    @sk.BilinearForm
    def helm(u, v, w):
        return w.c * ddot(grad(u), grad(v)) + w.s * dot(u, v)

    K = sk.asm(helm, b, c=g["c"], s=g["s"])
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL
    # the device geometry tabulation reproduces the reference bit for bit
    assert np.array_equal(b.dx, g["dx"])
    assert np.array_equal(b.tabulated_gradients, g["grads"])


def p2_basis(g, quadrature=None):
    m = sk.MeshTet2(g["p"], g["t"])
    return sk.Basis(m, sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=quadrature)


def test_p2_mesh_from_mesh_first_seen():
    g = load_golden("p2_aniso")
    m2 = sk.MeshTet2.from_mesh(sk.MeshTet(g["pj"], g["t0"]))
    assert np.array_equal(m2.t, g["t"]) and np.array_equal(m2.p, g["p"])


def test_p2_anisotropic_fused():
    g = load_golden("p2_aniso")
    b = p2_basis(g, (g["X"], g["W"]))
    assert b.is_affine
    E, Q = b._coefficient_shape
    Apub = np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    K = sk.asm(aniso, b, A=Apub)
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL
    Ans = np.broadcast_to(np.moveaxis(g["Ans"], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    Kn = sk.asm(aniso, b, A=Ans)
    assert relerr(Kn.data, g["ns_data"]) < RTOL
    # native (E,Q,3,3) layout and materialised per-point copies give the same
    Knat = sk.asm(aniso, b, A=np.ascontiguousarray(np.broadcast_to(g["A"][:, None], (E, Q, 3, 3))))
    assert relerr(Knat.data, g["data"]) < RTOL
    # geometry tabulated on the device matches the reference bit for bit
    assert np.array_equal(b.dx, g["dx"]) and np.array_equal(b.tabulated_gradients, g["grads"])
    assert np.array_equal(b._geometry_determinants, g["det"])


def test_p2_anisotropic_per_point_tabulated_path():
    g = load_golden("p2_aniso")
    b = p2_basis(g, (g["X"], g["W"]))
    E, Q = b._coefficient_shape
    rng = np.random.default_rng(11)
    Aq = np.broadcast_to(g["A"][:, None], (E, Q, 3, 3)) * (1 + 0.1 * rng.random((E, Q, 1, 1)))
    K = sk.asm(aniso, b, A=Aq)
    ob = O.make_basis(g["p"], g["t"], True, quadrature=(g["X"], g["W"]))
    data, indptr, indices = O.cross_gradient_tensor_assemble(ob, O.anisotropic_tensor(Aq, (E, Q)))
    assert np.array_equal(K.indices, indices)
    assert relerr(K.data, data) < RTOL


def test_p2_laplace_with_an_order_6_rule():
    """intorder above 4 selects the collapsed Gauss-Legendre rule (basis.py:1580-1598): 125 points for order
    6; P2 Laplace with it against the reference's own output (fixture simplex_rules).  The rule is compared
    to 1e-15: numpy's Gauss-Legendre weights on an Arm host differ from the fixture's x86 values in the
    last bits."""
    g = load_golden("simplex_rules")
    b = sk.Basis(sk.MeshTet2(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP2(), dim=1), intorder=6)
    assert b.X.shape == (3, 125)
    assert relerr(b.X, g["X6"]) < 1e-15 and relerr(b.W, g["W6"]) < 1e-15
    K = sk.asm(lap, b)
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL


def test_curved_p2_geometry_takes_the_tabulated_path():
    """Edge nodes moved off their edges' midpoints make the quadratic map curved (isoparametric, all ten
    nodes: basis.py:2194-2294): the basis is not affine and every form runs the tabulated kernels.
    Geometry bit for bit, Laplace and anisotropic diffusion against the reference's own outputs (fixture
    p2_curved); mass and load on scalar P2, elasticity on vector P2 and P1 on the ten-node mesh (which
    keeps the quadratic geometry map, basis.py:2274-2283) against the oracle."""
    g = load_golden("p2_curved")
    p, t = g["p"], g["t"]
    m = sk.MeshTet2(p, t)
    XW = (g["X"], g["W"])
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=XW)
    assert not b.is_affine
    assert np.array_equal(b.dx, g["dx"]) and np.array_equal(b.tabulated_gradients, g["grads"])
    assert np.array_equal(b._geometry_determinants, g["det"]) and np.array_equal(b.global_coordinates, g["xq"])
    ob = O.make_basis(p, t, True, quadrature=XW)
    E, Q = b._coefficient_shape

    K = sk.asm(lap, b)
    assert np.array_equal(K.indptr, g["lap_indptr"]) and np.array_equal(K.indices, g["lap_indices"])
    assert relerr(K.data, g["lap_data"]) < RTOL
    Apub = np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    Ka = sk.asm(aniso, b, A=Apub)
    same_pattern(Ka, g)
    assert relerr(Ka.data, g["data"]) < RTOL

    @sk.BilinearForm
    def mass(u, v, w):
        return dot(u, v)

    @sk.LinearForm
    def load(v, w):
        return dot(w.f, v)

    assert relerr(sk.asm(mass, b).data, O.bilinear_assemble(ob, value=1.0)[0]) < RTOL
    f = 1.0 + np.sin(3.0 * ob.x[..., 0]) * ob.x[..., 1]
    assert relerr(sk.asm(load, b, f=f), O.linear_assemble(ob, value=f[..., None])) < RTOL

    @sk.BilinearForm
    def elasticity(u, v, w):
        return 2.0 * ddot(sym_grad(u), sym_grad(v)) + 10.0 * div(u) * div(v)

    bv = sk.Basis(m, sk.ElementVector(sk.ElementTetP2(), dim=3), quadrature=XW)
    obv = O.make_basis(p, t, True, comp=3, quadrature=XW)
    Kv = sk.asm(elasticity, bv)
    dv, indptr_v, indices_v = O.bilinear_assemble(obv, symmetric_gradient=2.0, divergence=10.0)
    assert np.array_equal(Kv.indptr, indptr_v) and np.array_equal(Kv.indices, indices_v)
    assert relerr(Kv.data, dv) < RTOL

    b1 = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=XW)
    assert not b1.is_affine
    ob1 = O.make_basis(p, t, False, quadrature=XW)
    assert np.array_equal(b1.dx, ob1.dx)
    K1 = sk.asm(lap, b1)
    d1, indptr1, indices1 = O.bilinear_assemble(ob1, gradient=1.0)
    assert np.array_equal(K1.indptr, indptr1) and np.array_equal(K1.indices, indices1)
    assert relerr(K1.data, d1) < RTOL


def test_p2_constant_tensor_combined_with_isotropic_term_and_rejections():
    """The reference's anisotropic-form cases (tests/test_anisotropic_forms.py:41-125) on P2 tets against
    its own outputs (fixture aniso_forms_p2): a constant (3, 3) tensor gives a symmetric matrix; a
    nonsymmetric tensor summed with an isotropic mass term; a scalar coefficient with a unit axis reads as
    (E, Q) (_coefficients.py:84); a tensor of the wrong shape raises ValueError and a vector field
    UnsupportedNativeForm, with the reference's messages."""
    g = load_golden("aniso_forms_p2")
    b = p2_basis(g, (g["X"], g["W"]))
    E, Q = b._coefficient_shape

    K = sk.asm(aniso, b, A=g["A_const"])
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL
    assert abs(K - K.T).max() <= 2e-14 * np.max(np.abs(K.data))

    @sk.BilinearForm
    def aniso_mass(u, v, w):
        return dot(mul(w.A, grad(u)), grad(v)) + 0.25 * dot(u, v)

    Kc = sk.asm(aniso_mass, b, A=g["A_nonsym"])
    Kc.sort_indices()
    assert np.array_equal(Kc.indptr, g["combined_indptr"]) and np.array_equal(Kc.indices, g["combined_indices"])
    assert relerr(Kc.data, g["combined"]) < RTOL
    assert abs(Kc - Kc.T).max() > 1e-3 * np.max(np.abs(Kc.data))

    @sk.BilinearForm
    def kmass(u, v, w):
        return w.k * dot(u, v)

    k = g["k"]
    for raw in (k, k[..., None], k[None]):
        assert relerr(sk.asm(kmass, b, k=raw).data, g["kmass"]) < RTOL

    with pytest.raises(ValueError, match="recommended scikit-fem shape"):
        sk.asm(aniso, b, A=np.eye(2))
    vb = sk.Basis(sk.MeshTet2(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP2(), dim=3),
                  quadrature=(g["X"], g["W"]))
    with pytest.raises(sk.UnsupportedNativeForm, match="scalar field"):
        sk.asm(aniso, vb, A=np.eye(3))


@pytest.mark.parametrize("precision", ["fp64", "fp64_emulated"])
def test_p2_fp64_class_paths(precision):
    """Native FP64 and the double-float (FP32-pair) path both meet the FP64 bar."""
    g = load_golden("p2_aniso")
    b = p2_basis(g, (g["X"], g["W"]))
    E, Q = b._coefficient_shape
    Apub = np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    K = sk.asm(aniso, b, A=Apub, precision=precision)
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL
    Ans = np.broadcast_to(np.moveaxis(g["Ans"], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    assert relerr(sk.asm(aniso, b, A=Ans, precision=precision).data, g["ns_data"]) < RTOL


@pytest.mark.parametrize("precision", ["fp64_emulated", "split_fp32"])
def test_p1_reduced_paths(precision):
    g = load_golden("p1_laplace")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X1, W1))
    Kk = sk.asm(klap, b, kappa=g["kappa"][:, None], precision=precision)
    assert relerr(Kk.data, g["kdata"]) < (RTOL if precision == "fp64_emulated" else 1e-7)


def test_emulated_path_handles_extreme_scales():
    """A mesh scaled by 1e-50 leaves FP32 range: the emulated path must still
    return FP64-accurate values (it falls back to FP64)."""
    g = load_golden("p1_laplace")
    for scale in (1e-50, 1e40):
        b = sk.Basis(sk.MeshTet(g["p"] * scale, g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=1),
                     quadrature=(X1, W1))
        K = sk.asm(lap, b, precision="fp64_emulated")
        assert relerr(K.data / scale, g["data"]) < RTOL


def test_p2_split_precision_error_bound():
    g = load_golden("p2_aniso")
    b = p2_basis(g, (g["X"], g["W"]))
    E, Q = b._coefficient_shape
    Apub = np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    K = sk.asm(aniso, b, A=Apub, precision="split_fp32")
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < 1e-7


def test_p2_laplace_default_keast_rule():
    g = load_golden("p2_laplace_default")
    b = p2_basis(g)
    K = sk.asm(lap, b)
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL


def test_n1_maxwell():
    g = load_golden("n1_maxwell")
    nb = sk.AffineTetN1Basis(sk.MeshTet(g["p"], g["t"]))
    assert np.array_equal(nb.dof_map.topology.edges, g["edges"])
    assert np.array_equal(nb.element_dofs, g["element_edges"])
    assert np.array_equal(nb.basis_signs, g["signs"])
    asmb = sk.TetN1Assembler(nb)
    K = asmb.assemble_maxwell(mass_coefficient=1.0, curl_coefficient=(1.0 / g["mu"])[:, None])
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL
    # per-point coefficients through the explicit quadrature loop
    Q = len(nb.W)
    Kp = asmb.assemble_maxwell(mass_coefficient=np.ones((nb.mesh.nelements, Q)),
                               curl_coefficient=np.repeat((1.0 / g["mu"])[:, None], Q, 1)
                               * (1 + 0 * np.arange(Q))[None])
    assert relerr(Kp.data, g["data"]) < RTOL


def test_n1_split_precision_error_bound():
    """Split-FP32 element contraction (FP64 geometry and slot sums): <= 1e-7
    relative to the reference's FP64 matrix."""
    g = load_golden("n1_maxwell")
    nb = sk.AffineTetN1Basis(sk.MeshTet(g["p"], g["t"]))
    asmb = sk.TetN1Assembler(nb)
    K = asmb.assemble_maxwell(mass_coefficient=1.0, curl_coefficient=(1.0 / g["mu"])[:, None], precision="split_fp32")
    same_pattern(K, g)
    err = relerr(K.data, g["data"])
    assert 0 < err < 1e-7


def test_n1_vector_load():
    """TetN1LinearAssembler.assemble_vector_load vs the reference (array and callable fields)."""
    g = load_golden("n1_load")
    nb = sk.AffineTetN1Basis(sk.MeshTet(g["p"], g["t"]))
    la = sk.TetN1LinearAssembler(nb)
    assert relerr(nb.global_coordinates, g["xq"]) < 1e-15
    r = la.assemble_vector_load(g["f"])
    assert relerr(r, g["load"]) < RTOL
    r2 = la.assemble_vector_load(lambda x: np.stack([np.sin(3.0 * x[0]), x[1] * x[2], np.cos(2.0 * x[2]) - x[0]]))
    assert r2 is r  # reused vector, as the reference's
    assert relerr(r2, g["load_callable"]) < RTOL
    with pytest.raises(ValueError, match="vector load must broadcast"):
        la.assemble_vector_load(np.ones((2, 3)))


def test_n1_mass_and_curl_separately():
    g = load_golden("n1_maxwell")
    nb = O.make_n1_basis(g["p"], g["t"])
    gb = sk.AffineTetN1Basis(sk.MeshTet(g["p"], g["t"]))
    a = sk.TetN1Assembler(gb)
    E, Q = nb.dx.shape
    Km = a.assemble_mass(2.0).copy()
    Kc = a.assemble_curl_curl().copy()
    dm, _, _ = O.n1_assemble_maxwell(nb, 2.0, 0.0)
    dc, _, _ = O.n1_assemble_maxwell(nb, 0.0, 1.0)
    assert relerr(Km.data, dm) < RTOL and relerr(Kc.data, dc) < RTOL


def test_n1_pointwise_coefficients_reused_matrix_and_contract():
    """The reference's TetN1Assembler cases (tests/test_hcurl_tet_assembler.py:51-95): a coefficient that
    varies over the quadrature points (the pointwise kernel) against the oracle, mass and curl-curl
    overwriting one matrix object, the memory estimate and budget, the basis type and coefficient shape
    errors, and thread limits that leave the values unchanged."""
    g = load_golden("n1_maxwell")
    nb = O.make_n1_basis(g["p"], g["t"])
    gb = sk.AffineTetN1Basis(sk.MeshTet(g["p"], g["t"]))
    a = sk.TetN1Assembler(gb)
    assert gb.dx.shape == nb.dx.shape
    coef = np.linspace(0.5, 1.5, gb.dx.size).reshape(gb.dx.shape)
    Km = a.assemble_mass(coef)
    ident = (id(Km), id(Km.data), id(Km.indices), id(Km.indptr))
    dm, indptr, indices = O.n1_assemble_maxwell(nb, coef, 0.0)
    assert np.array_equal(Km.indptr, indptr) and np.array_equal(Km.indices, indices)
    assert relerr(Km.data, dm) < RTOL
    Kc = a.assemble_curl_curl(coef)
    assert (id(Kc), id(Kc.data), id(Kc.indices), id(Kc.indptr)) == ident
    dc, _, _ = O.n1_assemble_maxwell(nb, 0.0, coef)
    assert relerr(Kc.data, dc) < RTOL
    Kmx = a.assemble_maxwell(mass_coefficient=coef, curl_coefficient=coef[::-1])
    dmx, _, _ = O.n1_assemble_maxwell(nb, coef, coef[::-1])
    assert relerr(Kmx.data, dmx) < RTOL

    est = sk.estimate_tet_n1_assembly_memory(gb)
    assert est.kind == "hcurl_tet_n1" and est.row_local_dofs == est.column_local_dofs == 6
    with pytest.raises(TypeError, match="AffineTetN1Basis"):
        sk.TetN1Assembler(sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=1)))
    with pytest.raises(sk.AssemblyMemoryBudgetError):
        sk.TetN1Assembler(gb, memory_limit_bytes=1)
    with pytest.raises(ValueError, match="mass coefficient"):
        a.assemble_mass(np.zeros((2, 2, 2)))
    with pytest.raises(ValueError, match="curl coefficient"):
        a.assemble_curl_curl(np.zeros(gb.dx.shape[0] + 1))

    with sk.thread_limit(1):
        serial = a.assemble_maxwell(mass_coefficient=1.3, curl_coefficient=0.2).data.copy()
    with sk.thread_limit(4):
        parallel = a.assemble_maxwell(mass_coefficient=1.3, curl_coefficient=0.2).data.copy()
    assert np.array_equal(serial, parallel)
    d13, _, _ = O.n1_assemble_maxwell(nb, 1.3, 0.2)
    assert relerr(serial, d13) < RTOL


def test_named_coefficient_components_use_the_first_axis():
    """The reference's coefficient-component cases (tests/test_coefficient_components.py:25-138, on
    scalar P1 tets; composite elements are outside this path) against its own outputs (fixture
    components_p1): components of a keyword array are taken along its first axis in bilinear and linear
    forms, beside an anisotropic tensor term; a missing parameter, an out-of-range component and a
    non-integer index raise the reference's messages."""
    g = load_golden("components_p1")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=1))
    assert np.array_equal(b.X, g["X"]) and np.array_equal(b.W, g["W"])
    E, Q = b.dx.shape

    @sk.BilinearForm
    def form(u, v, w):
        return (w.material[0] * dot(u, v) + w.material[1] * ddot(grad(u), grad(v))
                + dot(mul(w.diffusion, grad(u)), grad(v)))

    K = sk.asm(form, b, material=g["material"], diffusion=g["diffusion"])
    K.sort_indices()
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL

    @sk.LinearForm
    def load(v, w):
        return dot(w.loads[1], v)

    assert relerr(sk.asm(load, b, loads=g["loads"]), g["r"]) < RTOL

    @sk.BilinearForm
    def indexed(u, v, w):
        return w.material[2] * dot(u, v)

    @sk.BilinearForm
    def noninteger(u, v, w):
        return w.material["stiffness"] * dot(u, v)

    with pytest.raises(ValueError, match="missing form parameter 'material'"):
        sk.asm(indexed, b)
    with pytest.raises(ValueError, match="has no component 2"):
        sk.asm(indexed, b, material=np.ones((2, E, Q)))
    with pytest.raises(ValueError, match="component index must be an integer"):
        sk.asm(noninteger, b)


def test_vector_p1_elasticity_terms():
    g = load_golden("vp1_elasticity")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(X1, W1))

    @sk.BilinearForm
    def elast(u, v, w):
        return 2.0 * ddot(sym_grad(u), sym_grad(v)) + 10.0 * div(u) * div(v) + 0.5 * dot(u, v)

    K = sk.asm(elast, b)
    same_pattern(K, g)
    assert relerr(K.data, g["data"]) < RTOL


def test_vector_tensor_tabulated_abi():
    """Full (E,Q,3,3,3,3) tensor through the C ABI (the neo-Hookean tangent layout)."""
    import torch

    from skfemntv_gb300 import _device as dev
    from skfemntv_gb300._native import call
    from skfemntv_gb300.assembly import Pattern

    g = load_golden("nh_vp1")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(X1, W1))
    ob = O.make_basis(g["p"], g["t"], False, comp=3, quadrature=(X1, W1))
    A = O.nh_tangent(O.displacement_gradient(ob, g["u"]), 1.0, 10.0)
    E, Q = b._coefficient_shape
    pat = Pattern(b._dev_dofs(), b._dev_dofs(), E, 12, 12, b.N, b.N)
    vals = dev.empty(pat.nnz, np.float64)
    tab = b._device_tabulation()
    call("skg_h1_assemble_tensor_tabulated", pat.h, dev.ptr(b._dev_dofs()), E, 4, 3, Q, dev.ptr(tab["grad"]),
         dev.ptr(tab["dx"]), dev.ptr(dev.to_device(A, np.float64)), dev.ptr(vals), None, dev.stream_ptr())
    torch.cuda.synchronize()
    indptr, indices = pat.host_csr()
    assert np.array_equal(indices, g["indices"])
    assert relerr(vals.cpu().numpy(), g["data"]) < RTOL


def test_p2_load_vector():
    g = load_golden("p2_load")
    b = p2_basis(g, (g["X"], g["W"]))

    @sk.LinearForm
    def load(v, w):
        return dot(w.f, v)

    r = sk.asm(load, b, f=g["f"])
    assert relerr(r, g["rhs"]) < RTOL


def test_repeatable_bits():
    g = load_golden("p2_aniso")
    b = p2_basis(g, (g["X"], g["W"]))
    E, Q = b._coefficient_shape
    Apub = np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    d1 = sk.asm(aniso, b, A=Apub).data.copy()
    d2 = sk.asm(aniso, b, A=Apub).data.copy()
    assert np.array_equal(d1.view(np.int64), d2.view(np.int64))


def test_geometry_errors_match_reference():
    flat = sk.MeshTet(np.array([[0., 1., 0., 0.], [0., 0., 1., 0.], [0., 0., 0., 0.]]), np.array([[0], [1], [2], [3]]))
    with pytest.raises(ValueError, match="cell=0, quadrature_point=0.*near_singular_or_non_finite"):
        sk.Basis(flat, sk.ElementVector(sk.ElementTetP1(), dim=1))
    tiny = sk.MeshTet(np.array([[0., 1., 0., 0.], [0., 0., 1., 0.], [0., 0., 0., 1.]]) * 1e-50,
                      np.array([[0], [1], [2], [3]]))
    b = sk.Basis(tiny, sk.ElementVector(sk.ElementTetP1(), dim=1))
    assert b.geometry_diagnostics.minimum_determinant > 0
    bad = sk.MeshTet(np.eye(3, 4), np.array([[0], [1], [1], [2]]))
    with pytest.raises(ValueError, match="repeats a corner"):
        sk.AffineTetN1Basis(bad)


def test_geometry_validation_cases_match_reference():
    """The reference's tetrahedral geometry checks (tests/test_geometry_validation.py:22-137, its tet cases
    and the tet analogue of its triangle condition-number case): the diagnostics of a valid mesh, one
    uniformly inverted tet accepted and reported, a 1e-50-scaled tet accepted with its determinant, an
    edge node that inverts a quadratic tet inside rejected at the first quadrature point where the
    determinant turns negative, and the Frobenius condition number of a flat but valid tet."""
    scalar = sk.ElementVector(sk.ElementTetP1(), dim=1)
    mesh = sk.MeshTet()
    b = sk.Basis(mesh, scalar)
    d = b.geometry_diagnostics
    Q = b.X.shape[1]
    assert isinstance(d, sk.GeometryDiagnostics)
    assert d.element_count == mesh.nelements and d.quadrature_points_per_element == Q
    assert d.minimum_determinant > 0 and d.maximum_determinant >= d.minimum_determinant
    assert d.minimum_scaled_determinant > 0 and d.determinant_tolerance > 0
    assert 0 <= d.worst_element < mesh.nelements and 0 <= d.worst_quadrature_point < Q
    assert d.maximum_condition_number >= 3
    assert 0 <= d.worst_condition_element < mesh.nelements and 0 <= d.worst_condition_quadrature_point < Q

    inverted = sk.MeshTet(np.array([[0., 0., 1., 0.], [0., 1., 0., 0.], [0., 0., 0., 1.]]),
                          np.array([[0], [1], [2], [3]]))
    b = sk.Basis(inverted, scalar)
    assert b.geometry_diagnostics.maximum_determinant < 0
    assert b.geometry_diagnostics.minimum_scaled_determinant == pytest.approx(1.0)
    assert b.geometry_diagnostics.negative_orientation_elements == 1
    assert np.all(b.dx > 0)

    scale = 1e-50
    b = sk.Basis(sk.MeshTet(scale * sk.MeshTet().p, sk.MeshTet().t), scalar)
    np.testing.assert_allclose(b.geometry_diagnostics.minimum_determinant, scale ** 3, rtol=2e-15)
    assert b.geometry_diagnostics.minimum_scaled_determinant == pytest.approx(1.0)

    m2 = sk.MeshTet2.from_mesh(sk.MeshTet())
    points = m2.p.copy()
    points[:, 4] = -2.0
    corner = points[:, m2.t[:4, 0]]
    assert np.linalg.det(corner[:, 1:] - corner[:, :1]) > 0
    with pytest.raises(ValueError, match=r"cell=0, quadrature_point=2, determinant=-.*reason=orientation_change"):
        sk.Basis(sk.MeshTet2(points, m2.t), sk.ElementVector(sk.ElementTetP2(), dim=1), intorder=4)

    flat = sk.MeshTet(np.array([[0., 1., 0., 0.], [0., 0., 1., 0.], [0., 0., 0., 1e-8]]),
                      np.array([[0], [1], [2], [3]]))
    d = sk.Basis(flat, scalar).geometry_diagnostics
    assert d.maximum_condition_number == pytest.approx(np.sqrt((2 + 1e-16) * (2 + 1e16)))
    assert d.worst_condition_element == 0 and d.worst_condition_quadrature_point == 0


def test_full_size_p1_laplace_vs_oracle():
    """The 32^3 x 6 Laplace configuration, compared entry by entry."""
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, 33),) * 3)
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X1, W1))
    K = sk.asm(lap, b)
    assert K.nnz == 513313
    ob = O.make_basis(m.p, m.t, False, quadrature=(X1, W1))
    data, indptr, indices = O.bilinear_assemble(ob, gradient=1.0)
    assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
    assert relerr(K.data, data) < RTOL


def test_device_resident_csr_handoff():
    """assemble_torch returns the same matrix as a CUDA sparse CSR tensor."""
    import torch
    from skfemntv_gb300.assembly import NativeTensorForm

    g = load_golden("p2_aniso")
    b = p2_basis(g, (g["X"], g["W"]))
    E, Q = b._coefficient_shape
    Apub = np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    form = NativeTensorForm(b)
    K = form.assemble(Apub, copy=True)
    assert relerr(K.data, g["data"]) < RTOL
    T = form.assemble_torch(Apub)
    x = np.random.default_rng(0).standard_normal(K.shape[1])
    y = (T @ torch.as_tensor(x, device="cuda")[:, None]).cpu().numpy()[:, 0]
    assert relerr(y, K @ x) < 1e-13
    gn = load_golden("n1_maxwell")
    a = sk.TetN1Assembler(sk.AffineTetN1Basis(sk.MeshTet(gn["p"], gn["t"])))
    Kn = a.assemble_maxwell(mass_coefficient=1.0).copy()
    Tn = a.assemble_maxwell_torch(mass_coefficient=1.0)
    xn = np.random.default_rng(1).standard_normal(Kn.shape[1])
    yn = (Tn @ torch.as_tensor(xn, device="cuda")[:, None]).cpu().numpy()[:, 0]
    assert relerr(yn, Kn @ xn) < 1e-13


@pytest.mark.parametrize("exponent", [-980, 1000])
def test_p2_exact_rule_entries_far_from_unit_scale(exponent):
    """The FP64 exact-rule element pass forms most entries from shared sums
    with the factors 2, 4 and 8 applied to the exponent bits; when a G entry's
    exponent leaves the range where that is exact, the element takes one
    table evaluation per entry instead.  A coefficient scaled by 2^-980 puts
    G there; one scaled by 2^1000 keeps G just inside the range, near the top
    (every value stays normal and finite, and a power-of-two scaling is
    exact): the result is the golden matrix scaled the same way."""
    g = load_golden("p2_aniso")
    b = p2_basis(g, (g["X"], g["W"]))
    E, Q = b._coefficient_shape
    scale = 2.0 ** exponent
    Apub = np.broadcast_to(np.moveaxis(g["A"] * scale, (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    K = sk.asm(aniso, b, A=Apub)
    same_pattern(K, g)
    assert relerr(K.data / scale, g["data"]) < RTOL


def _asymmetry_cases():
    """Per-element tensors around the symmetry tolerance |A_kl - A_lk| <=
    1e-14 (|A_00| + |A_11| + |A_22| + |A_01| + |A_02| + |A_12|)."""
    base = np.array([[2.0, 0.3, 0.1], [0.3, 1.5, 0.2], [0.1, 0.2, 1.2]])
    size = np.abs(base[np.triu_indices(3)]).sum()
    cases = {"exact": base.copy()}
    a = base.copy()
    a[1, 0] = np.nextafter(np.nextafter(np.nextafter(a[0, 1], 1.0), 1.0), 1.0)  # 3 units in the last place
    cases["ulps"] = a
    a = base.copy()
    a[0, 2], a[2, 0] = 1e-20, -1e-20  # opposite signs, far inside the tolerance
    cases["tiny_opposite"] = a
    a = base.copy()
    a[0, 1], a[1, 0] = 0.0, -0.0
    cases["signed_zeros"] = a
    a = base.copy()
    a[2, 1] = a[1, 2] + 0.9e-14 * size  # inside, beyond what the bit test accepts
    cases["inside"] = a
    a = base.copy()
    a[2, 1] = a[1, 2] + 1.1e-14 * size
    cases["outside"] = a
    a = base.copy()
    a[1, 0] = a[0, 1] * (1 + 2.0 ** -40)
    cases["outside_relative"] = a
    return cases


def _symmetric_to_tolerance(A):
    scale = 1e-14 * (abs(A[0, 0]) + abs(A[1, 1]) + abs(A[2, 2]) + abs(A[0, 1]) + abs(A[0, 2]) + abs(A[1, 2]))
    return bool(abs(A[0, 1] - A[1, 0]) <= scale and abs(A[0, 2] - A[2, 0]) <= scale
                and abs(A[1, 2] - A[2, 1]) <= scale)


@pytest.mark.parametrize("precision", ["fp64", "fp64_emulated", "split_fp32"])
def test_p2_coefficient_symmetry_decision(precision):
    """The element pass mirrors the upper triangle exactly when the element's
    tensor is symmetric to 1e-14 of its size (a bit-level test first, the
    floating-point test when that one fails; the same decision).  One tet per
    case: the assembled 10 x 10 matrix is exactly symmetric where mirrored;
    in FP64 an unmirrored one shows its tensor's asymmetry."""
    from skfemntv_gb300.assembly import NativeTensorForm

    g = load_golden("p2_aniso")
    m = sk.MeshTet(np.array([[0.0, 1.0, 0.1, 0.2], [0.0, 0.1, 0.9, 0.3], [0.0, 0.2, 0.1, 1.1]]),
                   np.array([[0], [1], [2], [3]]))
    b = sk.Basis(sk.MeshTet2.from_mesh(m), sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(g["X"], g["W"]))
    form = NativeTensorForm(b)
    for name, A in _asymmetry_cases().items():
        expect = _symmetric_to_tolerance(A)
        assert expect == (name not in ("outside", "outside_relative")), name
        K = form.assemble(np.broadcast_to(A[:, :, None, None], (3, 3, 1, 4)), precision=precision).toarray()
        mirrored = bool(np.array_equal(K, K.T))
        if expect:
            assert mirrored, (precision, name)
        elif precision == "fp64":
            assert not mirrored, name


def _mixed_orientation_meshes():
    axis = np.linspace(0.0, 1.0, 3)
    original = sk.MeshTet.init_tensor(axis, axis, axis)
    conn = original.t.copy()
    sel = np.arange(original.nelements) % 2 == 0
    first = conn[0, sel].copy()
    conn[0, sel] = conn[1, sel]
    conn[1, sel] = first
    return original, sk.MeshTet(original.p, conn)


def test_n1_orientation_invariance():
    """As the reference's test_hcurl_tet_robustness.py:31-77: swapping two vertices of
    every other tetrahedron (inverting it) leaves the Maxwell operator and the
    vector load unchanged up to the edge permutation."""
    original_mesh, mixed_mesh = _mixed_orientation_meshes()
    ob = sk.AffineTetN1Basis(original_mesh, intorder=4)
    mb = sk.AffineTetN1Basis(mixed_mesh, intorder=4)
    assert ob.geometry_diagnostics.inverted_cell_count == 0
    assert 0 < mb.geometry_diagnostics.inverted_cell_count < mixed_mesh.nelements
    lookup = {tuple(e): i for i, e in enumerate(mb.dof_map.topology.edges.T)}
    perm = np.array([lookup[tuple(e)] for e in ob.dof_map.topology.edges.T])
    Ko = sk.TetN1Assembler(ob).assemble_maxwell(mass_coefficient=1.3, curl_coefficient=0.2).toarray()
    Km = sk.TetN1Assembler(mb).assemble_maxwell(mass_coefficient=1.3, curl_coefficient=0.2).toarray()[perm][:, perm]
    np.testing.assert_allclose(Ko, Km, atol=4e-13)

    def field(x):
        return np.array((1.0 + x[1], x[0] * x[2], -0.25 + x[0] * x[1]))

    lo = sk.TetN1LinearAssembler(ob).assemble_vector_load(field).copy()
    lm = sk.TetN1LinearAssembler(mb).assemble_vector_load(field)[perm]
    np.testing.assert_allclose(lo, lm, atol=4e-14)


def test_cross_assemble_kinds_matches_reference():
    """NativeCrossBilinearForm.assemble_kinds (bilinear_form.py:244-334) on vector P1: the four value /
    gradient pairings with a per-point coefficient of both signs against the reference's own outputs
    (fixture cross_kinds); an unknown kind, normal_gradient without facet normals and mismatched
    component counts raise ValueError."""
    g = load_golden("cross_kinds")
    m = sk.MeshTet(g["p"], g["t"])
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(g["X"], g["W"]))
    assert b.nelems == m.nelements == b.dx.shape[0]
    form = sk.NativeCrossBilinearForm(b, b)
    assert form.test_normals is None and form.trial_normals is None
    for row in ("value", "gradient"):
        for column in ("value", "gradient"):
            K = form.assemble_kinds(row, column, g["c"])
            key = f"{row}_{column}_"
            assert np.array_equal(K.indptr, g[key + "indptr"]) and np.array_equal(K.indices, g[key + "indices"])
            assert relerr(K.data, g[key + "data"]) < RTOL, (row, column)
    with pytest.raises(ValueError, match="cross kind must be"):
        form.assemble_kinds("curl", "value")
    with pytest.raises(ValueError, match="requires test-basis normals"):
        form.assemble_kinds("normal_gradient", "value")
    bs = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(g["X"], g["W"]))
    with pytest.raises(ValueError, match="matching components"):
        sk.NativeCrossBilinearForm(b, bs).assemble_kinds("value", "value")


def test_cross_basis_assembly_matches_reference():
    """Two-basis asm (Stokes-type coupling div(v) u, a weighted P2 x P1 mass) and
    NativeCrossBilinearForm.assemble_tensor (gradient and value tensors on vector
    P1) against the reference's own outputs."""
    g = load_golden("cross")
    m = sk.MeshTet(g["p0"], g["t0"])
    m2 = sk.MeshTet2.from_mesh(m)
    XW = (g["X"], g["W"])
    bv2 = sk.Basis(m2, sk.ElementVector(sk.ElementTetP2(), dim=3), quadrature=XW)
    bs1 = sk.Basis(m2, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=XW)
    bs2 = sk.Basis(m2, sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=XW)

    @sk.BilinearForm
    def coupling(u, v, w):
        return div(v) * u

    @sk.BilinearForm
    def cmass(u, v, w):
        return w.c * dot(u, v)

    def check(K, prefix):
        assert K.shape == tuple(g[f"{prefix}_shape"])
        assert np.array_equal(K.indptr, g[f"{prefix}_indptr"]) and np.array_equal(K.indices, g[f"{prefix}_indices"])
        assert relerr(K.data, g[f"{prefix}_data"]) < RTOL

    check(sk.asm(coupling, bs1, bv2), "b")
    check(sk.asm(cmass, bs1, bs2, c=g["c"]), "m")
    bvp1 = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=XW)
    cf = sk.NativeCrossBilinearForm(bvp1, bvp1)
    check(cf.assemble_tensor("gradient", "gradient", g["T6"]), "t")
    check(cf.assemble_tensor("value", "value", g["Tv"]), "v")
    with pytest.raises(ValueError, match="tensor coefficient must broadcast"):
        cf.assemble_tensor("gradient", "gradient", np.ones((2, 2)))
    with pytest.raises(ValueError, match="row divergence requires"):
        cf.assemble("row_divergence", 1.0)


@pytest.mark.parametrize("element,cells", [("p1", 16), ("p2", 16), ("p2", 28)])
@pytest.mark.parametrize("precision", ["fp64", "fp64_emulated", "split_fp32"])
def test_host_output_matches_device(element, cells, precision):
    """The host-output path writes exactly the values of the device path: one
    copy after the passes for small outputs (16^3), and at 28^3 (5.1 M values,
    above the chunking threshold) the element and row passes interleaved over
    16 row chunks, each chunk's values copied while later chunks run."""
    from skfemntv_gb300.assembly import NativeTensorForm

    g = load_golden("p2_aniso")
    axis = np.linspace(0.0, 1.0, cells + 1)
    m = sk.MeshTet.init_tensor(axis, axis, axis)
    if element == "p2":
        b = sk.Basis(sk.MeshTet2.from_mesh(m), sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(g["X"], g["W"]))
    else:
        b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(g["X"], g["W"]))
    E, Q = b._coefficient_shape
    M = np.random.default_rng(7).standard_normal((E, 3, 3))
    A = M @ np.swapaxes(M, 1, 2) + 3.0 * np.eye(3)
    Apub = np.broadcast_to(np.moveaxis(A, (1, 2), (0, 1))[..., None], (3, 3, E, Q))
    form = NativeTensorForm(b)
    assert form.pattern.row_groups  # the fixed-order row-group passes serve this pattern
    K = form.assemble(Apub, precision=precision, copy=True)
    D = form.assemble_device(Apub, precision=precision)[:K.nnz].cpu().numpy()
    assert np.array_equal(K.data.view(np.int64), D.view(np.int64))
    K2 = form.assemble(2.0 * Apub, precision=precision, copy=False)  # reused page-locked values
    assert np.allclose(K2.data, 2.0 * D, rtol=1e-14, atol=0)


@pytest.mark.parametrize("cells", [12, 34])
@pytest.mark.parametrize("precision", ["fp64", "split_fp32"])
def test_n1_host_output_matches_device(precision, cells):
    """N1 Maxwell through the host-output path (per-element curl coefficient
    read from host memory; at 34^3, 4.6 M values, copies per row chunk) equals
    the device path bit for bit."""
    axis = np.linspace(0.0, 1.0, cells + 1)
    mesh = sk.MeshTet.init_tensor(axis, axis, axis)
    asmb = sk.TetN1Assembler(sk.AffineTetN1Basis(mesh))
    assert asmb.pattern.row_groups
    nu = np.exp(np.random.default_rng(3).normal(0.0, 0.3, mesh.nelements))[:, None]
    K = asmb.assemble_maxwell(mass_coefficient=1.0, curl_coefficient=nu, precision=precision)
    D = asmb.assemble_maxwell_torch(mass_coefficient=1.0, curl_coefficient=nu, precision=precision)
    d = D.values().cpu().numpy()
    assert np.array_equal(K.data.view(np.int64), d.view(np.int64))


def test_fp64_rate_probe():
    """The FP64 roof the bench reports against: a positive FMA rate of the
    order of GB300's FP64 pipe (hundreds of GFMA/s)."""
    import ctypes
    from skfemntv_gb300._native import call

    rate = ctypes.c_double()
    call("skg_fp64_fma_rate", ctypes.byref(rate), None)
    assert 50.0 < rate.value < 50000.0


@pytest.mark.parametrize("scale", [1e40, 1e12, 1.0])
def test_n1_split_precision_extreme_scales(scale):
    """N1 split precision works in coordinates scaled by 2^-s and unscales in
    the FP64 exponent, so meshes far outside the FP32 range (coordinates up to
    1e40) stay within 1e-7 of the FP64 pass like a unit mesh.  (Tiny meshes are
    rejected as singular by the basis, as the reference's isclose(detJ, 0)
    check does, hcurl_basis.py:321-322.)"""
    axis = np.linspace(0.0, 1.0, 5)
    m = sk.MeshTet.init_tensor(axis, axis, axis)
    mesh = sk.MeshTet(m.p * scale, m.t)
    asmb = sk.TetN1Assembler(sk.AffineTetN1Basis(mesh))
    nu = np.exp(np.random.default_rng(4).normal(0.0, 0.3, mesh.nelements))[:, None]
    K64 = asmb.assemble_maxwell(mass_coefficient=1.0, curl_coefficient=nu).copy()
    Ks = asmb.assemble_maxwell(mass_coefficient=1.0, curl_coefficient=nu, precision="split_fp32")
    assert np.all(np.isfinite(Ks.data))
    assert relerr(Ks.data, K64.data) < 1e-7


KINDS = ("value", "gradient", "symmetric_gradient", "divergence")


@pytest.mark.parametrize("quadratic,comp", [(False, 1), (False, 3), (True, 1), (True, 3)])
@pytest.mark.parametrize("kinds", [KINDS, ("value",), ("symmetric_gradient", "divergence"), ("gradient",)])
def test_tabulated_kinds_per_point_coefficients(quadratic, comp, kinds):
    """Per-point coefficients of every kind on the default rules (4-point P1, 11-point Keast P2) through the
    tabulated kernels (symmetric element-per-thread kernel for P1 and scalar P2, row-band kernel for vector
    P2), against the oracle's BilinearFormAssembler restatement on a jittered mesh."""
    from skfemntv_gb300.assembly import NativeBilinearForm

    rng = np.random.default_rng(101 + 10 * quadratic + comp)
    n = 4
    m = sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, n + 1),) * 3)
    inner = np.all((m.p > 1e-9) & (m.p < 1 - 1e-9), axis=0)
    m.p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, (3, int(inner.sum())))
    if quadratic:
        m = sk.MeshTet2.from_mesh(m)
    elem = sk.ElementTetP2() if quadratic else sk.ElementTetP1()
    b = sk.Basis(m, sk.ElementVector(elem, dim=comp))
    E, Q = b._coefficient_shape
    co = {k: rng.uniform(0.5, 2.0, (E, Q)) for k in kinds}
    K = NativeBilinearForm(b).assemble(**co)
    ob = O.make_basis(m.p, m.t, quadratic, comp=comp)
    d, indptr, indices = O.bilinear_assemble(ob, **co)
    assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
    assert relerr(K.data, d) < RTOL


@pytest.mark.parametrize("comp", [1, 3])
@pytest.mark.parametrize("kinds", [KINDS, ("value", "gradient"), ("symmetric_gradient", "divergence")])
@pytest.mark.parametrize("one_point", [False, True])
def test_fused_p1_forms_per_element_coefficients(comp, kinds, one_point):
    """Affine P1 forms with per-element coefficients go through the fused kernel (no tabulated point data:
    the basis' tabulation is never built) and match the oracle, on the device and through the host matrix."""
    from skfemntv_gb300.assembly import NativeBilinearForm

    rng = np.random.default_rng(7 + comp + 10 * one_point + len(kinds))
    n = 5
    m = sk.MeshTet.init_tensor(*(np.linspace(0.0, 2.0, n + 1),) * 3)
    inner = np.all((m.p > 1e-9) & (m.p < 2 - 1e-9), axis=0)
    m.p[:, inner] += rng.uniform(-0.3 / n, 0.3 / n, (3, int(inner.sum())))
    quadrature = (X1, W1) if one_point else None
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=comp), quadrature=quadrature)
    E, Q = b._coefficient_shape
    co = {k: rng.uniform(0.5, 2.0, (E, 1)) for k in kinds}
    form = NativeBilinearForm(b)
    K = form.assemble(**co)
    assert b._tab is None  # fused path: no per-point tabulation
    ob = O.make_basis(m.p, m.t, False, comp=comp, quadrature=quadrature)
    d, indptr, indices = O.bilinear_assemble(ob, **co)
    assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
    assert relerr(K.data, d) < RTOL
    dv = form.assemble_device(**co).cpu().numpy()[: len(d)]
    assert np.array_equal(dv.view(np.int64), K.data.view(np.int64))
    # scalar constants take no array at all
    K2 = form.assemble(**{k: 1.5 for k in kinds}).data.copy()
    d2, _, _ = O.bilinear_assemble(ob, **{k: 1.5 for k in kinds})
    assert relerr(K2, d2) < RTOL


def test_fused_p1_forms_chunked_host_output():
    """Vector P1 elasticity above the chunking threshold (> 2^22 nnz): host values delivered in row chunks equal
    the device values bit for bit, and the per-point path (tabulated kernels) agrees to rounding."""
    import torch

    from skfemntv_gb300.assembly import NativeBilinearForm

    n = 32
    m = sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, n + 1),) * 3)
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=3))
    form = NativeBilinearForm(b)
    assert form.pattern.nnz > 1 << 22
    co = dict(value=0.5, symmetric_gradient=2.0, divergence=10.0)
    host = form.assemble(**co).data.copy()
    dv = form.assemble_device(**co).cpu().numpy()[: form.pattern.nnz]
    assert np.array_equal(host.view(np.int64), dv.view(np.int64))
    E, Q = b._coefficient_shape
    pts = {k: torch.full((E, Q), v, dtype=torch.float64, device="cuda") for k, v in co.items()}
    tab = form.assemble_device(**pts).cpu().numpy()[: form.pattern.nnz]
    assert b._tab is not None
    assert relerr(tab, dv) < RTOL


@pytest.mark.parametrize("rule", ["one_point", "vertices"])
def test_p2_anisotropic_fused_rule_not_exact_on_quadratics(rule):
    """P2 anisotropic diffusion through the fused FP64 path with a rule that does not integrate quadratics
    exactly: the element pass reads the rule's table (the exact-rule kernel with integer factors is not
    eligible), symmetric and nonsymmetric A, against the oracle on the reference's algorithm."""
    g = load_golden("p2_aniso")
    if rule == "one_point":
        X, W = X1, W1
    else:  # the four vertices with weight 1/24: exact on linears only
        X, W = np.array([[0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0]]), np.full(4, 1.0 / 24.0)
    b = p2_basis(g, (X, W))
    assert b.is_affine
    E, Q = b._coefficient_shape
    ob = O.make_basis(g["p"], g["t"], True, quadrature=(X, W))
    for key in ("A", "Ans"):
        Apub = np.broadcast_to(np.moveaxis(g[key], (1, 2), (0, 1))[..., None], (3, 3, E, Q))
        K = sk.asm(aniso, b, A=Apub)
        d, indptr, indices = O.cross_gradient_tensor_assemble(ob, O.anisotropic_tensor(Apub, (E, Q)))
        assert np.array_equal(K.indptr, indptr) and np.array_equal(K.indices, indices)
        assert relerr(K.data, d) < RTOL


def _numpy_diagnostics(det, tol, cond):
    """The reference's host reductions (python/skfemntv/basis.py:2296-2356)."""
    scaled = np.abs(det) / (tol / (64.0 * np.finfo(np.float64).eps))
    flat = int(np.argmin(scaled))
    cflat = int(np.argmax(cond))
    Q = det.shape[1]
    return dict(element_count=det.shape[0], quadrature_points_per_element=Q,
                minimum_determinant=float(np.min(det)), maximum_determinant=float(np.max(det)),
                minimum_scaled_determinant=float(scaled.flat[flat]), worst_element=flat // Q,
                worst_quadrature_point=flat % Q, determinant_tolerance=float(tol.flat[flat]),
                negative_orientation_elements=int(np.count_nonzero(det[:, 0] < 0.0)),
                maximum_condition_number=float(cond.flat[cflat]), worst_condition_element=cflat // Q,
                worst_condition_quadrature_point=cflat % Q)


@pytest.mark.parametrize("flip", [False, True])
def test_geometry_diagnostics_device_reduction(flip):
    """Basis.geometry_diagnostics reduces det / tol / cond on the device; every
    field equals the reference's numpy reductions over the same arrays,
    including the first-occurrence choice of the worst point."""
    g = load_golden("p2_aniso")
    t = g["t"].copy()
    if flip:  # every third element with vertices 1 and 2 (and the edge nodes) swapped: negative orientation
        sel = np.arange(t.shape[1]) % 3 == 0
        t[:, sel] = g["t"][[0, 2, 1, 3, 6, 5, 4, 7, 9, 8]][:, sel]
    b = sk.Basis(sk.MeshTet2(g["p"], t), sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(g["X"], g["W"]))
    d = b.geometry_diagnostics
    want = _numpy_diagnostics(b._geometry_determinants, b._geometry_tolerances, b._geometry_condition_numbers)
    for k, v in want.items():
        assert getattr(d, k) == v, (k, getattr(d, k), v)
    if not flip:
        assert d.minimum_determinant == float(np.min(g["det"]))
        assert d.maximum_condition_number == float(np.max(g["cond"]))
    else:
        assert 0 < d.negative_orientation_elements < t.shape[1]
