"""Host-side tests that need no GPU: the C ABI library loads and exports every
symbol declared in include/skfem_gb300.h, and the host logic of the drop-in
(form tracing, quadrature tables, mesh generation, DOF numbering, runtime
controls, memory preflight) matches the reference's behaviour."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
from conftest import ROOT, load_golden

import skfemntv_gb300 as sk
from skfemntv_gb300 import _native, quadrature
from skfemntv_gb300.basis import number_dofs
from skfemntv_gb300.forms import (Parameters, QuadratureValue, _Field, _LinearSum, _LinearTerm, _Sum, _Term,
                                  ddot, div, dot, grad, mul, sym_grad)


def header_symbols():
    text = open(os.path.join(ROOT, "include", "skfem_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(skg_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = _native.load()
    syms = header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s
        assert s in _native.SIGNATURES, f"{s} missing from the ctypes binding"
    assert lib.skg_version() >= 100


def header_parameter_counts():
    """Number of parameters of every function the header declares (comments stripped)."""
    text = open(os.path.join(ROOT, "include", "skfem_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"^(?:int|const char \*)\s*(skg_\w+)\(([^)]*)\);", text, re.M):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


def test_ctypes_signatures_match_header_parameter_counts():
    counts = header_parameter_counts()
    assert set(counts) == set(header_symbols())
    for name, n in counts.items():
        assert len(_native.SIGNATURES[name]) == n, (name, len(_native.SIGNATURES[name]), n)


def test_n1_basis_entry_points_check_arguments_before_device_work():
    """The N1 basis entry points reject empty rules, bad layouts and missing arrays with SKG_EINVAL and a
    message before any device call, and return at once for an empty mesh."""
    from skfemntv_gb300._native import call

    X = np.full((3, 1), 0.25)
    W = np.array([1.0 / 6.0])
    t = np.array([0.5])
    hX, hW, ht = (a.ctypes.data_as(ctypes.c_void_p) for a in (X, W, t))
    cases = [
        ("skg_n1_element_matrices", (None, 0, None, None, 1, 0, hX, hW, None, None, 0, 1, 1, None, None),
         "quadrature rule is empty"),
        ("skg_n1_element_matrices", (None, 0, None, None, 1, 1, hX, hW, None, None, 2, 1, 1, None, None),
         "coefficient layout"),
        ("skg_n1_element_matrices", (None, 0, None, None, 1, 1, hX, hW, None, None, 0, 1, 1, None, None),
         "mesh or output arrays are NULL"),
        ("skg_n1_evaluate", (None, 0, None, None, None, 1, 1, 0, hX, None, 0, None, None), "quadrature rule is empty"),
        ("skg_n1_evaluate", (None, 0, None, None, None, 1, 1, 1, hX, None, 0, None, None),
         "mesh, coefficient or output arrays are NULL"),
        ("skg_n1_edge_points", (None, 0, None, 1, 0, ht, None, None), "edge rule is empty"),
        ("skg_n1_edge_points", (None, 0, None, 1, 1, ht, None, None), "mesh, edge or output arrays are NULL"),
        ("skg_n1_edge_moments", (None, 0, None, 1, 1, None, None, None, None), "edge rule is empty"),
        ("skg_n1_edge_moments", (None, 0, None, 1, 1, hW, None, None, None),
         "mesh, edge, field or output arrays are NULL"),
    ]
    for name, args, message in cases:
        with pytest.raises(ValueError, match=message):
            call(name, *args)
    call("skg_n1_element_matrices", None, 0, None, None, 0, 1, hX, hW, None, None, 0, 1, 1, None, None)
    call("skg_n1_evaluate", None, 0, None, None, None, 0, 0, 1, hX, None, 0, None, None)
    call("skg_n1_edge_points", None, 0, None, 0, 1, ht, None, None)
    call("skg_n1_edge_moments", None, 0, None, 0, 1, hW, None, None, None)


def test_nvcc_targets_sm103a_only():
    import build_native

    assert build_native.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


# ---------------------------------------------------------------- forms

def _trial():
    return _Field("trial", "value")


def _test():
    return _Field("test", "value")


def test_form_terms():
    u, v = _trial(), _test()
    assert ddot(grad(u), grad(v)) == _Term("gradient", None, 1.0)
    assert dot(grad(u), grad(v)) == _Term("gradient", None, 1.0)  # accepted (reference raises)
    assert dot(u, v) == _Term("value", None, 1.0)
    assert ddot(sym_grad(u), sym_grad(v)) == _Term("symmetric_gradient", None, 1.0)
    assert div(u) * div(v) == _Term("divergence", None, 1.0)
    A = np.eye(3)
    t = dot(mul(A, grad(u)), grad(v))
    assert t.kind == "gradient_tensor" and np.array_equal(t.coefficient, A)
    s = 2.0 * ddot(grad(u), grad(v)) + dot(u, v) - dot(u, v)
    assert isinstance(s, _Sum) and [x.factor for x in s.terms] == [2.0, 1.0, -1.0]
    # cross-basis couplings (forms.py:407-486 of the reference)
    assert div(v) * u == _Term("row_divergence", None, 1.0)
    assert u * div(v) == _Term("row_divergence", None, 1.0)
    assert div(u) * v == _Term("column_divergence", None, 1.0)
    assert (2.0 * div(u)) * v == _Term("column_divergence", None, 2.0)


def test_coefficients_and_parameters():
    w = Parameters({"kappa": QuadratureValue(np.ones((5, 1)), "kappa")})
    u, v = _trial(), _test()
    t = w.kappa * ddot(grad(u), grad(v))
    assert t.kind == "gradient" and t.coefficient.shape == (5, 1)
    sym = w.missing * dot(u, v)
    assert sym.coefficient.name == "missing"
    f = dot(w.kappa, v)
    assert isinstance(f, _LinearTerm) and f.kind == "value"
    g = ddot(np.zeros((3, 3, 5, 1)), grad(v)) + dot(w.kappa, v)
    assert isinstance(g, _LinearSum)


def test_unsupported_forms_raise():
    u, v = _trial(), _test()
    with pytest.raises(sk.UnsupportedNativeForm):
        dot(grad(u), v)
    with pytest.raises(sk.UnsupportedNativeForm):
        mul(np.eye(3), u)
    with pytest.raises(sk.UnsupportedNativeForm):
        dot(mul(np.eye(3), grad(u)), grad(u))


def test_public_api_contract():
    """tests/test_public_api_contract.py:11-64: exports unique and resolvable, no solver policy exported, an
    unsupported form raises UnsupportedNativeForm with no fallback, and the reference's module paths for
    the edge topology and DOF map resolve."""
    assert len(sk.__all__) == len(set(sk.__all__))
    for name in sk.__all__:
        assert hasattr(sk, name), name
    assert not hasattr(sk, "solve") and not hasattr(sk, "condense")

    @sk.BilinearForm
    def unsupported(u, v, w):
        return u

    with pytest.raises(sk.UnsupportedNativeForm):
        sk.asm(unsupported, None)
    from skfemntv_gb300.edge_dof_map import build_oriented_edge_dof_map
    from skfemntv_gb300.edge_topology import build_oriented_edge_topology

    assert build_oriented_edge_topology is sk.build_oriented_edge_topology
    assert build_oriented_edge_dof_map is sk.build_oriented_edge_dof_map


def test_asm_rejects_foreign_forms():
    with pytest.raises(TypeError):
        sk.asm(object(), None)
    with pytest.raises(ValueError):
        sk.asm(sk.BilinearForm(lambda u, v, w: dot(u, v)), None, num_threads=0)


# ---------------------------------------------------------------- setup

def test_quadrature_tables_match_reference_rules():
    g1 = load_golden("p1_helmholtz")
    X, W = quadrature.tet_rule_p1()
    assert np.array_equal(X, g1["X"]) and np.array_equal(W, g1["W"])
    g2 = load_golden("p2_laplace_default")
    X, W = quadrature.tet_rule_p2()
    assert np.array_equal(X, g2["X"]) and np.array_equal(W, g2["W"])
    gn = load_golden("n1_maxwell")
    X, W = quadrature.duffy_rule(2)
    assert np.array_equal(X, gn["X"]) and np.array_equal(W, gn["W"])
    for quadratic in (False, True):
        s1, g1_ = quadrature.tabulate(X, quadratic)
        s2, g2_ = O.tabulate_reference(X, quadratic)
        assert np.array_equal(s1, s2) and np.array_equal(g1_, g2_)


def test_quadrature_validation():
    """The reference's invalid custom rules (tests/test_quadrature.py:184-199, for tetrahedra): points of the
    wrong dimension, weights of the wrong length, and non-finite points or weights raise ValueError; a
    valid rule comes back contiguous and unchanged."""
    with pytest.raises(ValueError, match="shape"):
        quadrature.validate((np.zeros((2, 3)), np.zeros(3)))
    with pytest.raises(ValueError, match="shape"):
        quadrature.validate((np.zeros((1, 2)), np.ones(2)))
    with pytest.raises(ValueError, match="weights must have shape"):
        quadrature.validate((np.zeros((3, 2)), np.ones(3)))
    with pytest.raises(ValueError, match="finite"):
        quadrature.validate((np.full((3, 1), np.nan), np.ones(1)))
    with pytest.raises(ValueError, match="finite"):
        quadrature.validate((np.zeros((3, 1)), np.array([np.inf])))
    X = np.asfortranarray(np.array([[0.25, 0.1], [0.25, 0.2], [0.25, 0.3]]))
    W = np.array([0.1, 0.05])
    Xv, Wv = quadrature.validate((X, W))
    assert Xv.flags.c_contiguous and np.array_equal(Xv, X) and np.array_equal(Wv, W)


def test_high_order_rules_match_the_reference_and_integrate_monomials():
    """Above order 4 the basis takes the collapsed Gauss-Legendre rule (basis.py:1580-1598): the same numbers
    as the reference's (fixture simplex_rules), and exact for every monomial x^a y^b z^c with a + b + c up
    to the order (tests/test_quadrature.py:44-65), whose integral over the unit tetrahedron is
    a! b! c! / (a + b + c + 3)!."""
    from math import factorial

    g = load_golden("simplex_rules")
    for order in (5, 6, 7, 8):
        X, W = quadrature.simplex_rule(order)
        assert np.array_equal(X, g[f"X{order}"]) and np.array_equal(W, g[f"W{order}"]), order
        for a in range(order + 1):
            for b in range(order + 1 - a):
                for c in range(order + 1 - a - b):
                    exact = factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + 3)
                    got = float(np.sum(W * X[0] ** a * X[1] ** b * X[2] ** c))
                    assert abs(got - exact) <= 1e-14 * max(exact, 1e-3), (order, a, b, c)


def test_n1_duffy_rules_match_the_reference():
    """The N1 basis's Duffy product rules (hcurl_basis.py:37-56), orders 1 to 8, are the reference's numbers
    (fixture n1_rules), and the oracle's restatement agrees."""
    g = load_golden("n1_rules")
    for order in range(1, 9):
        X, W = quadrature.duffy_rule(order)
        assert np.array_equal(X, g[f"X{order}"]) and np.array_equal(W, g[f"W{order}"]), order
        Xo, Wo = O.duffy_quadrature(order)
        assert np.array_equal(Xo, X) and np.array_equal(Wo, W), order


def test_rules_too_large_for_the_geometry_kernel_are_rejected_before_device_work():
    """A P2 rule of order 12 (512 points) needs more reference tables than one block's shared memory holds:
    UnsupportedNativeForm before anything reaches the device; order 11 (343 points) fits."""
    with pytest.raises(sk.UnsupportedNativeForm, match="512 points"):
        sk.Basis(sk.MeshTet2(), sk.ElementVector(sk.ElementTetP2(), dim=1), intorder=12)
    X, W = quadrature.simplex_rule(11)
    assert 8 * len(W) * (4 * 10 + 4 * 10 + 1) <= 227 * 1024


def test_mesh_init_tensor_matches_reference():
    g = load_golden("p1_laplace")
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, 5),) * 3)
    assert np.array_equal(m.p, g["p"]) and np.array_equal(m.t, g["t"])
    x = np.array([0.0, 0.3, 1.0])
    y = np.array([0.0, 0.5, 0.7, 1.0])
    z = np.array([0.0, 1.0])
    m2 = sk.MeshTet.init_tensor(x, y, z)
    p, t = O.mesh_tet_tensor(x, y, z)
    assert np.array_equal(m2.p, p) and np.array_equal(m2.t, t)


def test_dof_numbering_matches_oracle():
    g = load_golden("p2_aniso")
    for nodes, comp in ((10, 1), (4, 3), (4, 1)):
        conn = g["t"][:nodes]
        N, _, ed, _ = number_dofs(g["p"].shape[1], conn, comp)
        # oracle numbering (restated from basis.py:1749-1777)
        used = np.zeros(g["p"].shape[1], bool)
        used[conn] = True
        act = np.flatnonzero(used)
        assert N == len(act) * comp
        pos = np.full(g["p"].shape[1], -1)
        pos[act] = np.arange(len(act))
        nd = np.arange(N).reshape(-1, comp).T
        ref = nd[:, pos[conn]].transpose(2, 1, 0).reshape(conn.shape[1], nodes * comp).T
        assert np.array_equal(ed, ref)


def test_runtime_controls():
    assert sk.get_num_threads() >= 1
    with pytest.raises(ValueError):
        sk.set_num_threads(0)
    with pytest.raises(ValueError):
        sk.set_num_threads(True)
    before = sk.get_num_threads()
    with sk.thread_limit(1) as eff:
        assert eff == 1 and sk.get_num_threads() == 1
    assert sk.get_num_threads() == before


class _SizesMesh:
    def __init__(self, E):
        self.nelements = E


class _SizesBasis:
    """Stand-in with the sizes a memory estimate reads (no device arrays)."""

    def __init__(self, E, Q, nodes, comp, N):
        self.mesh = _SizesMesh(E)
        self.W = np.full(Q, 1.0 / Q)
        self._nodes, self._comp, self.N = nodes, comp, N
        self.element_dofs = np.zeros((nodes * comp, E), dtype=np.int64)
        self._tab = None


def test_memory_budget_error():
    est = sk.estimate_bilinear_memory(_SizesBasis(40, 4, 4, 1, 30))
    with pytest.raises(sk.AssemblyMemoryBudgetError, match="budget exceeded") as captured:
        sk.enforce_memory_budget(est, 100)
    assert captured.value.estimate == est and captured.value.required_bytes > 100
    assert captured.value.largest_allocation in str(captured.value) and "local_dofs=4x4" in str(captured.value)
    sk.enforce_memory_budget(est, 10 ** 9)
    sk.enforce_memory_budget(est, None)
    with pytest.raises(ValueError, match="positive"):
        sk.enforce_memory_budget(est, 0)
    with pytest.raises(TypeError, match="integer or None"):
        sk.enforce_memory_budget(est, 1.5e9)
    with pytest.raises(TypeError, match="integer or None"):
        sk.enforce_memory_budget(est, True)
    with pytest.raises(ValueError, match="memory_safety_factor"):  # checked even without a budget
        sk.enforce_memory_budget(est, None, safety_factor=0.5)
    assert issubclass(sk.AssemblyMemoryBudgetError, MemoryError)


def test_memory_estimate_counts_this_backends_allocations():
    """The reference's preflight contract (tests/test_memory_preflight.py:21-86) restated for the GPU
    backend: the fields keep their names and count the int32 device DOF maps and CSR, the float64 element
    matrices (E x Lr x Lc, as the reference's scatter map), the page-locked host matrix and one copy, the
    row incidence, and per-call staging.  A vector space scales the element matrices by 9; a cross
    estimate has its own kind and local sizes; what the basis already holds moves from the incremental
    bytes to basis_bytes, leaving the total unchanged."""
    E, Q, N = 96, 4, 60
    b = _SizesBasis(E, Q, 4, 1, N)
    est = sk.estimate_bilinear_memory(b)
    L = 4
    nnz = min(N * N, E * L * L)
    assert est.kind == "bilinear" and est.rows == est.columns == N
    assert est.nnz_upper_bound == nnz
    assert est.scatter_bytes == E * L * L * 8
    assert est.dof_map_bytes == E * L * 4 * 3  # the basis's device map and the pattern's two copies
    assert est.native_tabulation_bytes == E * Q * (4 * 4 + 7) * 8
    assert est.csr_bytes_upper_bound == 4 * (N + 1) + 12 * nnz + 2 * (12 * nnz + 8 * (N + 1))
    assert est.staging_bytes_upper_bound == 16 * 8 * E + 2 * 9 * E * Q * 8
    assert est.basis_bytes == b.element_dofs.nbytes + b.W.nbytes
    assert est.construction_peak_total_bytes_upper_bound > est.basis_bytes
    assert est.construction_peak_incremental_bytes_upper_bound > est.persistent_incremental_bytes_upper_bound
    assert "MiB" in sk.format_bytes(2 ** 20)

    vec = sk.estimate_bilinear_memory(_SizesBasis(E, Q, 4, 3, 3 * N))
    assert vec.row_local_dofs == 3 * est.row_local_dofs and vec.scatter_bytes == 9 * est.scatter_bytes
    assert vec.construction_peak_incremental_bytes_upper_bound > est.construction_peak_incremental_bytes_upper_bound

    cross = sk.estimate_bilinear_memory(_SizesBasis(E, Q, 4, 3, 3 * N), b)
    assert cross.kind == "cross-bilinear" and (cross.row_local_dofs, cross.column_local_dofs) == (12, 4)
    assert cross.scatter_bytes == E * 12 * 4 * 8
    with pytest.raises(ValueError, match="quadrature shapes must match"):
        sk.estimate_bilinear_memory(b, _SizesBasis(E, Q + 1, 4, 1, N))
    with pytest.raises(TypeError):
        sk.estimate_bilinear_memory(object())

    # once the basis holds its device map and tabulation they count as basis bytes
    b._dofs_dev = np.zeros((E, L), dtype=np.int32)
    b._tab = {"shape": np.zeros((E, Q, 4)), "grad": np.zeros((E, Q, 4, 3)), "dx": np.zeros((E, Q)),
              "x": np.zeros((E, Q, 3)), "det": np.zeros((E, Q)), "tol": np.zeros((E, Q)),
              "cond": np.zeros((E, Q))}
    held = sk.estimate_bilinear_memory(b)
    assert held.native_tabulation_bytes == 0 and held.dof_map_bytes == E * L * 4 * 2
    assert held.basis_bytes > est.basis_bytes
    assert held.construction_peak_total_bytes_upper_bound == est.construction_peak_total_bytes_upper_bound

    peak = est.construction_peak_total_bytes_upper_bound
    assert est.fits_in(peak, safety_factor=1.0) and not est.fits_in(peak, safety_factor=1.01)
    with pytest.raises(ValueError, match="at least 1"):
        est.fits_in(peak, safety_factor=0.9)


def test_no_product_module_imports_oracle():
    pkg = os.path.join(ROOT, "scikit-fem-native_gb300", "skfemntv_gb300")
    for f in os.listdir(pkg):
        if f.endswith(".py"):
            src = open(os.path.join(pkg, f)).read()
            assert "oracle" not in src.replace("oracle-free", ""), f


def test_bench_reference_arm_prints_the_contract_line():
    """bench.py --impl reference (the CPU oracle on the host cores) prints one JSON line with the GPU arm's
    metric, unit and config, a cpu_baseline describing the run and an e2e entry without host-device bytes."""
    import json
    import subprocess
    import sys

    import bench

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["value"] > 0 and d["steps"] == 1 and d["warmup"] >= 3
    assert d["config"]["workload"] == bench.CONFIG["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_coefficient_classification_routes_fused_and_tabulated_paths():
    """per_element decides between the fused per-element kernels and the tabulated per-point ones: a scalar
    stays 0-d, a coefficient constant over each element's points becomes (E,), one that varies gives None;
    shapes that do not broadcast to (E, Q) raise ValueError as the reference does."""
    from skfemntv_gb300.assembly import per_element, per_point

    E, Q = 5, 4
    assert np.ndim(per_element(2.5, E, Q, "value")) == 0
    c = np.arange(E, dtype=float)
    for form in (c[:, None], np.broadcast_to(c[:, None], (E, Q)), np.repeat(c[:, None], Q, axis=1)):
        got = per_element(form, E, Q, "value")
        assert got.shape == (E,) and np.array_equal(got, c)
    varying = np.arange(E * Q, dtype=float).reshape(E, Q)
    assert per_element(varying, E, Q, "value") is None
    assert per_point(varying, E, Q, "value").shape == (E, Q)
    assert per_point(1.0, E, Q, "value").shape == (E, Q)
    with pytest.raises(ValueError):
        per_element(np.ones((E + 1, Q)), E, Q, "value")
    with pytest.raises(ValueError):
        per_point(np.ones((E, Q + 1)), E, Q, "value")


def test_component_access_errors_raise_before_assembly():
    """A missing parameter, an out-of-range component and a non-integer component index raise the
    reference's ValueErrors (tests/test_coefficient_components.py:122-138) while the form is traced or
    its coefficients evaluated, before anything reaches a basis or the device."""
    @sk.BilinearForm
    def indexed(u, v, w):
        return w.material[2] * dot(u, v)

    @sk.BilinearForm
    def noninteger(u, v, w):
        return w.material["stiffness"] * dot(u, v)

    with pytest.raises(ValueError, match="missing form parameter 'material'"):
        sk.asm(indexed, None)
    with pytest.raises(ValueError, match="has no component 2"):
        sk.asm(indexed, None, material=np.ones((2, 3, 4)))
    with pytest.raises(ValueError, match="component index must be an integer"):
        sk.asm(noninteger, None)


def test_native_linear_form_coefficient_rules():
    """NativeLinearForm._coefficient (linear_form.py:91-107, tests/test_compatible_forms.py:14-24): a
    constant keeps its shape, anything else is broadcast to (E, Q, C[, 3]); only float64 is accepted
    (TypeError), and a shape that does not broadcast raises ValueError naming the target shape."""
    f = sk.NativeLinearForm._coefficient
    assert f("value", np.array([2.0]), (100, 3, 1)).shape == (1,)
    assert f("gradient", np.array([[3.0, 4.0, 5.0]]), (100, 3, 1, 3)).shape == (1, 3)
    assert f("value", np.ones((100, 3, 1)), (100, 3, 1)).shape == (100, 3, 1)
    assert f("value", np.ones((100, 1, 1)), (100, 3, 1)).shape == (100, 3, 1)
    assert f("value", None, (100, 3, 1)) is None
    with pytest.raises(TypeError, match="dtype float64"):
        f("value", np.array([2], dtype=np.int64), (100, 3, 1))
    with pytest.raises(ValueError, match=r"gradient coefficient must broadcast to \(100, 3, 1, 3\)"):
        f("gradient", np.ones((7, 3)), (100, 3, 1, 3))


def test_coefficient_evaluation_factor_and_squeeze():
    """A term's coefficient times its factor (_coefficients.py:71-86): a factor of 1 leaves a broadcast
    view uncopied; squeezing, as bilinear scalar terms do, reads (E, Q, 1) and (1, E, Q) as (E, Q)."""
    from skfemntv_gb300.forms import Coefficient, _evaluate

    E, Q = 6, 4
    kappa = np.arange(E * Q, dtype=float).reshape(E, Q)
    A = np.broadcast_to(np.eye(3)[..., None, None], (3, 3, E, Q))
    got = _evaluate(Coefficient("A"), {"A": A}, 1.0)
    assert got.shape == (3, 3, E, Q) and got.strides[2:] == (0, 0)
    assert np.array_equal(_evaluate(Coefficient("A"), {"A": A}, 2.0), 2.0 * A)
    assert _evaluate(None, {}, 0.25) == 0.25
    for raw in (kappa[..., None], kappa[None]):
        assert np.array_equal(_evaluate(Coefficient("k"), {"k": raw}, 1.0, squeeze=True), kappa)
        assert _evaluate(Coefficient("k"), {"k": raw}, 1.0).shape == raw.shape
    assert _evaluate(Coefficient("k"), {"k": kappa[:, :1]}, 3.0, squeeze=True).shape == (E, 1)


def test_anisotropic_tensor_layouts_and_shape_error():
    """The three tensor layouts the reference accepts (forms.py:377-404) give one (E, Q, 3, 3) view, a
    tensor constant over each element's points goes to the fused per-element path in its own layout, and
    any other shape raises the reference's ValueError naming the recommended shape."""
    from skfemntv_gb300.assembly import anisotropic_tensor, tensor_per_element

    E, Q = 4, 5
    rng = np.random.default_rng(2)
    Aq = rng.random((E, Q, 3, 3))
    public = np.ascontiguousarray(np.moveaxis(Aq, (2, 3), (0, 1)))
    assert np.array_equal(anisotropic_tensor(public, E, Q), Aq)
    assert np.array_equal(anisotropic_tensor(Aq, E, Q), Aq)
    A = rng.random((3, 3))
    assert np.array_equal(anisotropic_tensor(A, E, Q), np.broadcast_to(A, (E, Q, 3, 3)))
    assert tensor_per_element(Aq, E, Q) is None and tensor_per_element(public, E, Q) is None
    arr, kind = tensor_per_element(A, E, Q)
    assert kind == 1 and np.array_equal(arr, np.broadcast_to(A, (E, 3, 3)))
    Ae = rng.random((E, 3, 3))
    arr, kind = tensor_per_element(np.broadcast_to(Ae[:, None], (E, Q, 3, 3)), E, Q)
    assert kind == 1 and np.array_equal(arr, Ae)
    arr, kind = tensor_per_element(np.repeat(np.moveaxis(Ae, 0, -1)[..., None], Q, axis=3), E, Q)
    assert kind == 2 and np.array_equal(arr, np.moveaxis(Ae, 0, -1))
    for bad in (np.eye(2), np.ones((3, 3, E, Q + 1)), np.ones((E, Q, 3))):
        with pytest.raises(ValueError, match="recommended scikit-fem shape"):
            tensor_per_element(bad, E, Q)
        with pytest.raises(ValueError, match="recommended scikit-fem shape"):
            anisotropic_tensor(bad, E, Q)
