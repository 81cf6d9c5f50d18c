"""Pin the CPU oracle against outputs of the reference itself (tests/golden).

Index structures must match exactly; values are compared bit for bit where
the oracle keeps the reference's summation order (serial paths), otherwise to
1e-14 relative to the largest entry.
"""
import numpy as np
import pytest

import oracle as O
from conftest import load_golden

X1 = np.array([[.25], [.25], [.25]])
W1 = np.array([1 / 6])


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_mesh_generation_matches_reference():
    g = load_golden("p1_laplace")
    p, t = O.mesh_tet_tensor(*(np.linspace(0, 1, 5),) * 3)
    assert np.array_equal(p, g["p"]) and np.array_equal(t, g["t"])


def test_p2_mesh_first_seen_edges():
    g = load_golden("p2_aniso")
    p2, t2 = O.mesh_tet2_from_mesh(g["pj"], g["t0"])
    assert np.array_equal(t2, g["t"])
    assert np.array_equal(p2, g["p"])


def test_p1_laplace_bit_exact():
    g = load_golden("p1_laplace")
    b = O.make_basis(g["p"], g["t"], False, quadrature=(X1, W1))
    data, indptr, indices = O.bilinear_assemble(b, gradient=1.0)
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    assert np.array_equal(data, g["data"])
    kd, _, _ = O.bilinear_assemble(b, gradient=g["kappa"][:, None])
    assert np.array_equal(kd, g["kdata"])


def test_p1_helmholtz_default_rule():
    g = load_golden("p1_helmholtz")
    b = O.make_basis(g["p"], g["t"], False)
    assert np.array_equal(b.X, g["X"]) and np.array_equal(b.W, g["W"])
    assert np.array_equal(b.dx, g["dx"]) and np.array_equal(b.grad, g["grads"])
    data, indptr, indices = O.bilinear_assemble(b, value=g["s"], gradient=g["c"])
    assert np.array_equal(indices, g["indices"])
    assert rel(data, g["data"]) < 1e-14


def test_p2_aniso_cross_tensor():
    g = load_golden("p2_aniso")
    b = O.make_basis(g["p"], g["t"], True, quadrature=(g["X"], g["W"]))
    assert np.array_equal(b.dx, g["dx"]) and np.array_equal(b.grad, g["grads"])
    assert np.array_equal(b.det, g["det"]) and np.array_equal(b.cond, g["cond"])
    E, Q = b.dx.shape
    T = O.anisotropic_tensor(np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q)), (E, Q))
    data, indptr, indices = O.cross_gradient_tensor_assemble(b, T)
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    assert np.array_equal(data, g["data"])
    Tn = O.anisotropic_tensor(np.broadcast_to(np.moveaxis(g["Ans"], (1, 2), (0, 1))[..., None], (3, 3, E, Q)), (E, Q))
    dn, _, _ = O.cross_gradient_tensor_assemble(b, Tn)
    assert np.array_equal(dn, g["ns_data"])


def test_p2_curved_isoparametric():
    """Edge nodes off the edges' midpoints (fixture p2_curved): the ten-node geometry map bit for bit, the
    anisotropic tensor and Laplace matrices in the reference's summation order."""
    g = load_golden("p2_curved")
    b = O.make_basis(g["p"], g["t"], True, quadrature=(g["X"], g["W"]))
    assert np.array_equal(b.dx, g["dx"]) and np.array_equal(b.grad, g["grads"])
    assert np.array_equal(b.det, g["det"]) and np.array_equal(b.x, g["xq"])
    E, Q = b.dx.shape
    T = O.anisotropic_tensor(np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q)), (E, Q))
    data, indptr, indices = O.cross_gradient_tensor_assemble(b, T)
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    assert np.array_equal(data, g["data"])
    ld, lip, lind = O.bilinear_assemble(b, gradient=1.0)
    assert np.array_equal(lip, g["lap_indptr"]) and np.array_equal(lind, g["lap_indices"])
    assert np.array_equal(ld, g["lap_data"])


def test_p2_threaded_colored_close():
    g = load_golden("p2_aniso")
    b = O.make_basis(g["p"], g["t"], True, quadrature=(g["X"], g["W"]))
    E, Q = b.dx.shape
    T = O.anisotropic_tensor(np.broadcast_to(np.moveaxis(g["A"], (1, 2), (0, 1))[..., None], (3, 3, E, Q)), (E, Q))
    data, _, _ = O.cross_gradient_tensor_assemble(b, T, threads=4)
    assert rel(data, g["data"]) < 1e-14


def test_p2_laplace_default_keast():
    g = load_golden("p2_laplace_default")
    b = O.make_basis(g["p"], g["t"], True)
    assert np.array_equal(b.X, g["X"]) and np.array_equal(b.W, g["W"])
    data, indptr, indices = O.bilinear_assemble(b, gradient=1.0)
    assert np.array_equal(indices, g["indices"])
    assert np.array_equal(data, g["data"])


def test_n1_maxwell():
    g = load_golden("n1_maxwell")
    nb = O.make_n1_basis(g["p"], g["t"])
    assert np.array_equal(nb.edges, g["edges"])
    assert np.array_equal(nb.element_dofs, g["element_edges"])
    assert np.array_equal(nb.signs, g["signs"])
    assert np.array_equal(nb.detJ, g["detJ"])
    data, indptr, indices = O.n1_assemble_maxwell(nb, 1.0, (1.0 / g["mu"])[:, None])
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    assert rel(data, g["data"]) < 1e-14


def test_n1_element_matrices_evaluation_and_interpolation():
    """The oracle's N1 element matrices summed over the edge DOFs give the reference's Maxwell matrix;
    edge-moment interpolation of a constant field gives the moments of its tangents, and evaluating them
    gives the field back with zero curl (the reference's own interpolation test,
    tests/test_hcurl_tet_interpolation.py:12-29)."""
    g = load_golden("n1_maxwell")
    nb = O.make_n1_basis(g["p"], g["t"])
    el = O.n1_element_matrices(nb, 1.0, (1.0 / g["mu"])[:, None])
    dofs = nb.element_dofs.T
    K = np.zeros((nb.N, nb.N))
    np.add.at(K, (np.repeat(dofs, 6, axis=1).ravel(), np.tile(dofs, (1, 6)).ravel()), el.ravel())
    rows = np.repeat(np.arange(nb.N), np.diff(g["indptr"]))
    assert rel(K[rows, g["indices"]], g["data"]) < 1e-14
    mass = O.n1_element_matrices(nb, include_curl=False)
    curl = O.n1_element_matrices(nb, include_mass=False)
    assert rel(mass + curl, O.n1_element_matrices(nb)) < 1e-15
    constant = np.array((1.25, -0.5, 0.75))
    m = O.n1_interpolate_edge_moments(g["p"], nb.edges, lambda x: constant[:, None] + 0.0 * x)
    tangents = g["p"][:, nb.edges[1]] - g["p"][:, nb.edges[0]]
    np.testing.assert_allclose(m, constant @ tangents, atol=2e-15)
    np.testing.assert_allclose(O.n1_evaluate(nb, m), np.broadcast_to(constant[:, None, None], (3,) + nb.dx.shape),
                               atol=2e-14)
    np.testing.assert_allclose(O.n1_evaluate(nb, m, curl=True), 0.0, atol=2e-14)


def _n1_field(x):
    return np.stack([np.sin(3.0 * x[0]) + x[1], x[0] * x[2], np.cos(2.0 * x[2]) - x[0] * x[1]])


def test_n1_basis_against_the_reference():
    """The reference's element matrices, evaluation of a seeded edge field and its curl, and edge-moment
    interpolation (fixture n1_basis, 3rd-order rule) against the oracle."""
    g = load_golden("n1_basis")
    nb = O.make_n1_basis(g["p"], g["t"], intorder=3)
    assert np.array_equal(nb.X, g["X"]) and np.array_equal(nb.W, g["W"])
    assert rel(O.n1_element_matrices(nb, include_curl=False), g["mass"]) < 1e-14
    assert rel(O.n1_element_matrices(nb, include_mass=False), g["curl_curl"]) < 1e-14
    assert rel(O.n1_evaluate(nb, g["u"]), g["values"]) < 1e-14
    assert rel(O.n1_evaluate(nb, g["u"], curl=True), g["curls"]) < 1e-14
    assert rel(O.n1_interpolate_edge_moments(g["p"], nb.edges, _n1_field, 4), g["moments"]) < 1e-15


def test_n1_vector_load():
    g = load_golden("n1_load")
    b = O.make_n1_basis(g["p"], g["t"])
    assert rel(O.n1_vector_load(b, g["f"]), g["load"]) < 1e-14
    xq = O.n1_global_coordinates(g["p"], g["t"], b.X)
    assert rel(xq, g["xq"]) < 1e-15
    fx = np.stack([np.sin(3.0 * xq[0]), xq[1] * xq[2], np.cos(2.0 * xq[2]) - xq[0]])
    assert rel(O.n1_vector_load(b, fx), g["load_callable"]) < 1e-14


def test_vector_p1_elasticity_terms():
    g = load_golden("vp1_elasticity")
    b = O.make_basis(g["p"], g["t"], False, comp=3, quadrature=(X1, W1))
    shp = b.dx.shape
    data, indptr, indices = O.bilinear_assemble(
        b, symmetric_gradient=np.full(shp, 2.0), divergence=np.full(shp, 10.0), value=np.full(shp, 0.5))
    assert np.array_equal(indices, g["indices"])
    assert np.array_equal(data, g["data"])


def test_neo_hookean_pieces():
    g = load_golden("nh_vp1")
    b = O.make_basis(g["p"], g["t"], False, comp=3, quadrature=(X1, W1))
    Gu = O.displacement_gradient(b, g["u"])
    P = O.nh_first_piola(Gu, 1.0, 10.0)
    r = O.linear_assemble(b, gradient=P)
    assert rel(r, g["residual"]) < 1e-14
    A = O.nh_tangent(Gu, 1.0, 10.0)
    data, indptr, indices = O.cross_gradient_tensor_assemble(b, A)
    assert np.array_equal(indices, g["indices"])
    assert rel(data, g["data"]) < 1e-13


def test_p2_load_vector():
    g = load_golden("p2_load")
    b = O.make_basis(g["p"], g["t"], True, quadrature=(g["X"], g["W"]))
    r = O.linear_assemble(b, value=g["f"][..., None])
    assert np.array_equal(r, g["rhs"])


def test_repeated_corner_rejected():
    t = np.array([[0], [1], [1], [2]])
    with pytest.raises(ValueError, match="repeats a corner"):
        O.edge_topology(t)


def test_geometry_validation_messages():
    p = np.array([[0., 1., 0., 0.], [0., 0., 1., 0.], [0., 0., 0., 0.]])  # flat tet
    t = np.array([[0], [1], [2], [3]])
    with pytest.raises(O.GeometryError, match="cell=0, quadrature_point=0.*near_singular"):
        O.make_basis(p, t, False)
    # tiny but valid (scale-aware tolerance) is accepted
    ps = np.array([[0., 1., 0., 0.], [0., 0., 1., 0.], [0., 0., 0., 1.]]) * 1e-50
    b = O.make_basis(ps, t, False)
    assert b.det[0, 0] > 0


def test_compatible_volume_forms():
    """Fixture forms_vp1 (the reference's compatible-forms cases on vector P1): loads and bilinear forms
    with constant, coordinate and parameter coefficients."""
    g = load_golden("forms_vp1")
    b = O.make_basis(g["p"], g["t"], False, comp=3, quadrature=(g["X"], g["W"]))
    x = np.moveaxis(b.x, -1, 0)
    assert rel(O.linear_assemble(b, value=g["force"]), g["r_force"]) < 1e-14
    assert rel(O.linear_assemble(b, gradient=g["tensor"][:, :, 0, 0]), g["r_tensor"]) < 1e-14
    field = np.stack((1.0 + x[0], x[1] ** 2, -0.5 * x[2]), axis=0)
    assert rel(O.linear_assemble(b, value=np.moveaxis(field, 0, -1)), g["r_coordinate"]) < 1e-14
    data, indptr, indices = O.bilinear_assemble(b, value=1.0)
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    assert rel(data, g["data"]) < 1e-14
    assert rel(O.bilinear_assemble(b, symmetric_gradient=2.0 * 0.7, divergence=2.3)[0], g["elasticity"]) < 1e-14
    assert rel(O.bilinear_assemble(b, value=1.0 + x[0] ** 2)[0], g["weighted_mass"]) < 1e-14
    assert rel(O.bilinear_assemble(b, value=1.8 * (1.0 + x[0]))[0], g["scaled_mass"]) < 1e-14
    rd = O.bilinear_assemble(b, value=1.3 * (1.0 + x[0] ** 2), gradient=0.4 * np.exp(-x[1]))[0]
    assert rel(rd, g["reaction_diffusion"]) < 1e-14


def test_coefficient_components_and_anisotropic_forms():
    """Fixtures components_p1 (first-axis components beside a tensor term, a linear-form component) and
    aniso_forms_p2 (a constant tensor, a nonsymmetric one plus an isotropic mass term, a scalar
    coefficient with a unit axis)."""
    g = load_golden("components_p1")
    b = O.make_basis(g["p"], g["t"], False, quadrature=(g["X"], g["W"]))
    E, Q = b.dx.shape
    pd, indptr, indices = O.bilinear_assemble(b, value=g["material"][0], gradient=g["material"][1])
    td, _, _ = O.cross_gradient_tensor_assemble(b, O.anisotropic_tensor(g["diffusion"], (E, Q)))
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    assert rel(pd + td, g["data"]) < 1e-14
    assert rel(O.linear_assemble(b, value=g["loads"][1][..., None]), g["r"]) < 1e-14

    g = load_golden("aniso_forms_p2")
    b = O.make_basis(g["p"], g["t"], True, quadrature=(g["X"], g["W"]))
    E, Q = b.dx.shape
    d, indptr, indices = O.cross_gradient_tensor_assemble(b, O.anisotropic_tensor(g["A_const"], (E, Q)))
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    assert rel(d, g["data"]) < 1e-14
    tn, _, _ = O.cross_gradient_tensor_assemble(b, O.anisotropic_tensor(g["A_nonsym"], (E, Q)))
    md, _, _ = O.bilinear_assemble(b, value=0.25)
    assert np.array_equal(indptr, g["combined_indptr"]) and np.array_equal(indices, g["combined_indices"])
    assert rel(tn + md, g["combined"]) < 1e-14
    assert rel(O.bilinear_assemble(b, value=g["k"])[0], g["kmass"]) < 1e-14


def test_p2_laplace_with_an_order_6_rule():
    """Fixture simplex_rules: P2 Laplace with the reference's order-6 collapsed rule."""
    g = load_golden("simplex_rules")
    b = O.make_basis(g["p"], g["t"], True, quadrature=(g["X6"], g["W6"]))
    data, indptr, indices = O.bilinear_assemble(b, gradient=1.0)
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    assert rel(data, g["data"]) < 1e-14
