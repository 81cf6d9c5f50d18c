"""The Nedelec basis beyond assembly, on the GPU: element matrices, evaluation of edge fields and their
curls, edge-moment interpolation, the oriented edge topology and the edge DOF map, against the oracle
(same seeded inputs) and with the reference's own cases (tests/test_hcurl_tet_basis.py,
test_hcurl_tet_interpolation.py, test_hcurl_tet_robustness.py, test_edge_topology.py,
test_edge_dof_map.py)."""
import numpy as np
import pytest
from scipy.sparse import coo_matrix

import oracle as O
from conftest import load_golden

pytestmark = pytest.mark.gpu
sk = pytest.importorskip("skfemntv_gb300")

RTOL = 1e-12


def relerr(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def _cube(resolution):
    axis = np.linspace(0.0, 1.0, resolution + 1)
    return sk.MeshTet.init_tensor(axis, axis, axis)


def _golden_bases(intorder=2):
    g = load_golden("n1_maxwell")
    return (g, sk.AffineTetN1Basis(sk.MeshTet(g["p"], g["t"]), intorder=intorder),
            O.make_n1_basis(g["p"], g["t"], intorder=intorder))


def _scatter(basis, elements):
    """Element matrices summed into a CSR matrix over the edge DOFs (tests/test_hcurl_tet_basis.py:10-16)."""
    dofs = basis.element_dofs.T
    rows = np.repeat(dofs, 6, axis=1).ravel()
    cols = np.tile(dofs, (1, 6)).ravel()
    return coo_matrix((elements.ravel(), (rows, cols)), shape=(basis.N, basis.N)).tocsr()


def test_n1_element_matrices_match_oracle_and_assembly():
    g, gb, ob = _golden_bases(intorder=3)
    Mm, Mc = gb.element_mass_matrices(), gb.element_curl_curl_matrices()
    assert Mm.shape == Mc.shape == (gb.mesh.nelements, 6, 6)
    assert relerr(Mm, O.n1_element_matrices(ob, include_curl=False)) < RTOL
    assert relerr(Mc, O.n1_element_matrices(ob, include_mass=False)) < RTOL
    a = sk.TetN1Assembler(gb)
    Km = a.assemble_mass().copy()
    Kc = a.assemble_curl_curl().copy()
    assert relerr(_scatter(gb, Mm).toarray(), Km.toarray()) < 1e-13
    assert relerr(_scatter(gb, Mc).toarray(), Kc.toarray()) < 1e-13


def test_n1_basis_against_the_reference():
    """Fixture n1_basis, produced by the reference: element matrices, evaluation of a seeded edge field
    and its curl, and edge-moment interpolation of a smooth field (3rd-order rule)."""
    g = load_golden("n1_basis")
    b = sk.AffineTetN1Basis(sk.MeshTet(g["p"], g["t"]), intorder=3)
    # the rule comes from numpy's Gauss-Legendre nodes and weights, as the reference's does; numpy's weights
    # on an Arm host differ from the x86 values in the fixture in the last bits
    assert relerr(b.X, g["X"]) < 1e-15 and relerr(b.W, g["W"]) < 1e-15
    assert relerr(b.element_mass_matrices(), g["mass"]) < RTOL
    assert relerr(b.element_curl_curl_matrices(), g["curl_curl"]) < RTOL
    assert relerr(b.evaluate(g["u"]), g["values"]) < RTOL
    assert relerr(b.evaluate_curl(g["u"]), g["curls"]) < RTOL
    assert relerr(b.interpolate_edge_moments(_field, quadrature_order=4), g["moments"]) < 1e-14


def test_n1_element_matrices_per_point_coefficients_through_the_c_abi():
    """coef_per_point = 1: per-point mass and curl coefficients through the explicit quadrature loop."""
    from skfemntv_gb300 import _device as dev
    from skfemntv_gb300._native import call

    g, gb, ob = _golden_bases()
    E, Q = gb.dx.shape
    mass = np.linspace(0.5, 1.5, E * Q).reshape(E, Q)
    curl = mass[::-1].copy()
    out = dev.empty((E, 6, 6), np.float64)
    d_mass, d_curl = dev.to_device(mass, np.float64), dev.to_device(curl, np.float64)
    call("skg_n1_element_matrices", dev.ptr(gb.mesh._dev("p")), gb.mesh.p.shape[1], dev.ptr(gb._t4),
         dev.ptr(gb._signs_dev), E, Q, dev.hptr(gb.X), dev.hptr(gb.W), dev.ptr(d_mass), dev.ptr(d_curl), 1, 1, 1,
         dev.ptr(out), dev.stream_ptr())
    assert relerr(out.cpu().numpy(), O.n1_element_matrices(ob, mass, curl)) < RTOL


def test_n1_basis_layout_geometry_and_rejections():
    """tests/test_hcurl_tet_basis.py:24-35 and 67-85."""
    b = sk.AffineTetN1Basis(_cube(1), intorder=3)
    E, Q = b.mesh.nelements, len(b.W)
    assert b.values.shape == b.curls.shape == (6, 3, E, Q)
    assert b.dx.shape == (E, Q) and b.element_dofs.shape == (6, E)
    assert b.geometry_diagnostics.minimum_volume > 0 and b.geometry_diagnostics.inverted_cell_count >= 0
    np.testing.assert_allclose(np.sum(b.dx), 1.0)

    class _Triangles:
        t = np.zeros((3, 1), dtype=np.int64)

        def dim(self):
            return 2

    with pytest.raises(TypeError, match="tetrahedral mesh"):
        sk.AffineTetN1Basis(_Triangles())
    singular = sk.MeshTet(np.array(((0., 1., 0., 1.), (0., 0., 1., 1.), (0., 0., 0., 0.))),
                          np.array(((0,), (1,), (2,), (3,))))
    with pytest.raises(ValueError, match="nonsingular tetrahedra"):
        sk.AffineTetN1Basis(singular)
    measured = sk.AffineTetN1Basis(_cube(1)).geometry_diagnostics.maximum_aspect_ratio
    with pytest.raises(ValueError, match="aspect ratio exceeds"):
        sk.AffineTetN1Basis(_cube(1), max_aspect_ratio=0.99 * measured)
    with pytest.raises(ValueError, match="positive finite scalar"):
        sk.AffineTetN1Basis(_cube(1), max_aspect_ratio=np.inf)


def _field(x):
    return np.array((np.sin(3.0 * x[0]) + x[1], x[0] * x[2], np.cos(2.0 * x[2]) - x[0] * x[1]))


def test_n1_evaluate_and_interpolate_match_oracle():
    g, gb, ob = _golden_bases(intorder=4)
    u = np.random.default_rng(5).standard_normal(gb.N)
    assert relerr(gb.evaluate(u), O.n1_evaluate(ob, u)) < RTOL
    assert relerr(gb.evaluate_curl(u), O.n1_evaluate(ob, u, curl=True)) < RTOL
    for order in (1, 4, 7):
        m = gb.interpolate_edge_moments(_field, quadrature_order=order)
        assert relerr(m, O.n1_interpolate_edge_moments(g["p"], ob.edges, _field, order)) < 1e-14


def test_n1_interpolation_reproduces_a_constant_field_and_validates():
    """tests/test_hcurl_tet_interpolation.py:12-42."""
    b = sk.AffineTetN1Basis(_cube(2), intorder=3)
    constant = np.array((1.25, -0.5, 0.75))
    c = b.interpolate_edge_moments(lambda x: constant[:, None] + 0.0 * x)
    edges = b.dof_map.topology.edges
    expected = np.einsum("ie,i->e", b.mesh.p[:, edges[1]] - b.mesh.p[:, edges[0]], constant)
    np.testing.assert_allclose(c, expected, atol=2e-15)
    values = b.evaluate(c)
    np.testing.assert_allclose(values, np.broadcast_to(constant[:, None, None], values.shape), atol=2e-14)
    np.testing.assert_allclose(b.evaluate_curl(c), 0.0, atol=2e-14)

    b1 = sk.AffineTetN1Basis(_cube(1))
    with pytest.raises(TypeError, match="field must be callable"):
        b1.interpolate_edge_moments(np.ones(3))
    with pytest.raises(ValueError, match="positive integer"):
        b1.interpolate_edge_moments(lambda x: x, quadrature_order=0)
    with pytest.raises(ValueError, match="broadcastable"):
        b1.interpolate_edge_moments(lambda x: np.zeros((2, x.shape[1])))
    with pytest.raises(ValueError, match="coefficients must have shape"):
        b1.evaluate(np.zeros(b1.N + 1))


def test_n1_interpolation_converges_in_hcurl_norm():
    """tests/test_hcurl_tet_interpolation.py:45-66: L2 and curl errors fall at least at rate 0.8."""
    def field(x):
        return np.array((0.0 * x[0], x[0] * x[2], x[0] * x[1]))

    def exact_curl(x):
        return np.array((0.0 * x[0], -x[1], x[2]))

    errors = []
    for resolution in (1, 2, 4):
        b = sk.AffineTetN1Basis(_cube(resolution), intorder=4)
        c = b.interpolate_edge_moments(field, quadrature_order=4)
        ve = b.evaluate(c) - field(b.global_coordinates)
        ce = b.evaluate_curl(c) - exact_curl(b.global_coordinates)
        l2 = np.sqrt(np.einsum("ieq,ieq,eq->", ve, ve, b.dx))
        cl2 = np.sqrt(np.einsum("ieq,ieq,eq->", ce, ce, b.dx))
        errors.append((l2, cl2, np.hypot(l2, cl2)))
    errors = np.asarray(errors)
    assert np.all(errors[1:] < errors[:-1])
    rates = np.log(errors[:-1] / errors[1:]) / np.log(2.0)
    assert np.all(rates > 0.8), rates


def _mixed_orientation_meshes():
    original = _cube(2)
    conn = original.t.copy()
    sel = np.arange(original.nelements) % 2 == 0
    first = conn[0, sel].copy()
    conn[0, sel] = conn[1, sel]
    conn[1, sel] = first
    return original, sk.MeshTet(original.p, conn)


def test_mixed_orientation_preserves_interpolant_and_error_norms():
    """tests/test_hcurl_tet_robustness.py:31-77: inverting every other tetrahedron leaves the
    interpolation coefficients (up to the edge permutation) and the error norms unchanged."""
    def field(x):
        return np.array((1.0 + x[1], x[0] * x[2], -0.25 + x[0] * x[1]))

    def exact_curl(x):
        return np.array((x[0], -x[1], -1.0 + 0.0 * x[2]))

    bases = [sk.AffineTetN1Basis(m, intorder=4) for m in _mixed_orientation_meshes()]
    lookup = {tuple(e): i for i, e in enumerate(bases[1].dof_map.topology.edges.T)}
    perm = np.array([lookup[tuple(e)] for e in bases[0].dof_map.topology.edges.T])
    c0 = bases[0].interpolate_edge_moments(field)
    c1 = bases[1].interpolate_edge_moments(field)[perm]
    np.testing.assert_allclose(c0, c1, atol=3e-15)
    norms = []
    for b in bases:
        c = b.interpolate_edge_moments(field)
        ve = b.evaluate(c) - field(b.global_coordinates)
        ce = b.evaluate_curl(c) - exact_curl(b.global_coordinates)
        norms.append((np.einsum("ieq,ieq,eq->", ve, ve, b.dx), np.einsum("ieq,ieq,eq->", ce, ce, b.dx)))
    np.testing.assert_allclose(norms[0], norms[1], atol=3e-14)


def _assert_local_orientation(t, topo):
    """Each directed local edge is its global edge, reversed where its sign is -1
    (tests/test_edge_topology.py:11-18)."""
    for cell in range(t.shape[1]):
        for local, (start, end) in enumerate(topo.local_edges):
            directed = (int(t[start, cell]), int(t[end, cell]))
            edge = tuple(int(v) for v in topo.edges[:, topo.element_edges[local, cell]])
            assert directed == (edge if topo.element_edge_signs[local, cell] == 1 else edge[::-1])


def test_edge_topology_and_dof_map_contracts():
    """tests/test_edge_topology.py:21-79 and test_edge_dof_map.py:14-76 on tetrahedra: unique ascending
    global edges, local orientation signs, numbering equal to the oracle's first-seen one, vertex
    reordering keeping the edge set, local/global coefficient round trips (a shared edge gives every cell
    the same moment), and the shape and repeated-corner errors."""
    from skfemntv_gb300.edge_dof_map import build_oriented_edge_dof_map
    from skfemntv_gb300.edge_topology import build_oriented_edge_topology

    one = sk.MeshTet()
    topo = build_oriented_edge_topology(one)
    assert topo.element_edges.shape == (6, 1)
    assert len(set(map(tuple, topo.edges.T))) == topo.edges.shape[1] == 6
    _assert_local_orientation(one.t, topo)

    cube = _cube(2)
    reordered = sk.MeshTet(cube.p, cube.t[[1, 0, 2, 3]])
    tops = [build_oriented_edge_topology(m) for m in (cube, reordered)]
    for m, t in zip((cube, reordered), tops):
        assert set(np.unique(t.element_edge_signs)) <= {-1, 1}
        assert np.all(t.edges[0] < t.edges[1])
        _assert_local_orientation(m.t, t)
        edges, ee, sg = O.edge_topology(m.t)
        assert np.array_equal(t.edges, edges) and np.array_equal(t.element_edges, ee)
        assert np.array_equal(t.element_edge_signs, sg)
    assert set(map(tuple, tops[0].edges.T)) == set(map(tuple, tops[1].edges.T))

    for m in (cube, reordered):
        dofs = build_oriented_edge_dof_map(m)
        assert dofs.ndofs == dofs.topology.edges.shape[1]
        values = np.array([10.0 * a + b for a, b in dofs.topology.edges.T])
        recovered = dofs.global_moments_from_local(dofs.local_coefficients(values))
        np.testing.assert_array_equal(recovered, values[dofs.element_dofs])
    counts = np.bincount(dofs.element_dofs.ravel(), minlength=dofs.ndofs)
    shared = int(np.flatnonzero(counts >= 2)[0])
    ordinal = np.arange(1.0, dofs.ndofs + 1.0)
    recovered = dofs.global_moments_from_local(dofs.local_coefficients(ordinal))
    for local, cell in np.argwhere(dofs.element_dofs == shared):
        assert recovered[local, cell] == ordinal[shared]
    with pytest.raises(ValueError, match="global edge coefficients"):
        dofs.local_coefficients(np.zeros((dofs.ndofs, 1)))
    with pytest.raises(ValueError, match="local edge coefficients"):
        dofs.global_moments_from_local(np.zeros(dofs.ndofs))

    class _RepeatedCorner:
        t = np.array([[0], [0], [1], [2]], dtype=np.int64)

        @staticmethod
        def dim():
            return 3

    with pytest.raises(ValueError, match="cell 0 repeats a corner vertex"):
        build_oriented_edge_topology(_RepeatedCorner())


def test_n1_on_a_quadratic_mesh_uses_its_corners():
    """A ten-node mesh gives the same edges and matrices as its corner mesh (hcurl_basis.py:295-306: the
    basis reads the four corner rows only)."""
    cube = _cube(2)
    b4 = sk.AffineTetN1Basis(cube)
    b10 = sk.AffineTetN1Basis(sk.MeshTet2.from_mesh(cube))
    assert np.array_equal(b4.dof_map.topology.edges, b10.dof_map.topology.edges)
    K4 = sk.TetN1Assembler(b4).assemble_maxwell(mass_coefficient=1.3, curl_coefficient=0.2).copy()
    K10 = sk.TetN1Assembler(b10).assemble_maxwell(mass_coefficient=1.3, curl_coefficient=0.2)
    assert np.array_equal(K4.indices, K10.indices) and np.array_equal(K4.data, K10.data)
