"""The allocation-free assembly entry point, called through the C ABI.

Callers that cannot let a library allocate device memory (their own pool
allocator owns the GPU, or they re-assemble inside a loop where cudaMalloc /
cudaFree is not allowed) use skg_h1_assemble_affine_noalloc, whose scratch is
a fixed static device array.  Its results must equal those of the ordinary
entry point skg_h1_assemble_affine, call after call (the array keeps the
previous call's contents, so a second call checks that nothing leaks from the
first).  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
sk = pytest.importorskip("skfemntv_gb300")

from skfemntv_gb300 import _device as dev  # noqa: E402
from skfemntv_gb300._native import SKG_FP64, SKG_FP64_EMULATED, SKG_SPLIT_FP32, load  # noqa: E402
from skfemntv_gb300.assembly import Pattern  # noqa: E402

RTOL = 1e-12
MAX_ELEMENTS = 262144


def _rule4():
    a, b = 0.5854101966249685, 0.1381966011250105
    return np.array([[a, b, b, b], [b, a, b, b], [b, b, a, b]]), np.full(4, 1.0 / 24.0)


def _tensors(E, rng, scale=1.0):
    A = rng.standard_normal((3, 3, E))
    A = np.ascontiguousarray(np.einsum("ije,kje->ike", A, A) + 3.0 * np.eye(3)[:, :, None]) * scale
    return dev.to_device(A, np.float64)


def _problem(n, quadratic, seed, scale=1.0, coef_scale=1.0):
    rng = np.random.default_rng(seed)
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    p = m.p.copy()
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
    mesh = sk.MeshTet(p * scale, m.t)
    if quadratic:
        mesh = sk.MeshTet2.from_mesh(mesh)
    X, W = _rule4()
    elem = sk.ElementTetP2() if quadratic else sk.ElementTetP1()
    basis = sk.Basis(mesh, sk.ElementVector(elem, dim=1), quadrature=(X, W))
    return mesh, basis, X, W, _tensors(mesh.nelements, rng, coef_scale)


def _fan(k, seed):
    """k tetrahedra sharing vertex 0, their other vertices all distinct: row 0
    of the P1 matrix has 3k + 1 columns, beyond the row-group records' 255,
    so both entry points take the per-row global-memory pass."""
    rng = np.random.default_rng(seed)
    p = np.hstack([np.zeros((3, 1)), rng.uniform(-1.0, 1.0, size=(3, 3 * k))])
    t = np.vstack([np.zeros(k, dtype=np.int64), np.arange(1, 3 * k + 1).reshape(k, 3).T])
    mesh = sk.MeshTet(p, t)
    X, W = _rule4()
    basis = sk.Basis(mesh, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X, W))
    return mesh, basis, X, W, _tensors(k, rng)


def _assemble(name, pat, mesh, basis, X, W, dA, precision, out):
    lib = load()
    L = basis._nodes
    args = [pat.h, dev.ptr(mesh._dev("p")), mesh.p.shape[1], dev.ptr(mesh._dev("t")), L, mesh.nelements,
            len(W), dev.hptr(X), dev.hptr(W), 2, dev.ptr(dA), precision, dev.ptr(out), dev.stream_ptr()]
    status = getattr(lib, name)(*args)
    torch.cuda.synchronize()
    return status


def _compare(mesh, basis, X, W, dA, precision, rtol, blocked=True):
    L = basis._nodes
    dofs = basis._dev_dofs()
    pat = Pattern(dofs, dofs, mesh.nelements, L, L, basis.N, basis.N)
    assert pat.row_groups == blocked
    ref = dev.empty(max(1, pat.nnz), np.float64)
    got = dev.empty(max(1, pat.nnz), np.float64)
    assert _assemble("skg_h1_assemble_affine", pat, mesh, basis, X, W, dA, precision, ref) == 0
    for call in range(2):  # two calls in a row share the static scratch array
        got.fill_(float("nan"))
        assert _assemble("skg_h1_assemble_affine_noalloc", pat, mesh, basis, X, W, dA, precision, got) == 0
        r, g = ref[: pat.nnz].cpu().numpy(), got[: pat.nnz].cpu().numpy()
        assert np.all(np.isfinite(g)), call
        if pat.nnz:
            assert np.max(np.abs(g - r)) <= rtol * np.max(np.abs(r)), call


@pytest.mark.parametrize("quadratic,precision", [(False, SKG_FP64), (True, SKG_FP64), (True, SKG_FP64_EMULATED),
                                                 (False, SKG_SPLIT_FP32), (True, SKG_SPLIT_FP32)])
def test_no_alloc_matches_allocating_entry_point(quadratic, precision):
    rtol = 1e-7 if precision == SKG_SPLIT_FP32 else RTOL
    _compare(*_problem(5 if quadratic else 8, quadratic, 3), precision, rtol)


@pytest.mark.parametrize("precision", [SKG_FP64_EMULATED, SKG_SPLIT_FP32])
def test_no_alloc_mesh_far_from_unit_scale(precision):
    """A mesh scaled by 1e40: the FP32-pair modes work in coordinates rescaled
    by a power of two, so both entry points stay in their mode (each within
    the mode's accuracy of the other)."""
    rtol = 1e-7 if precision == SKG_SPLIT_FP32 else RTOL
    _compare(*_problem(4, True, 5, scale=1e40), precision, rtol)


@pytest.mark.parametrize("precision", [SKG_FP64_EMULATED, SKG_SPLIT_FP32])
def test_no_alloc_out_of_fp32_range_falls_back_to_fp64(precision):
    """A coefficient scaled by 1e40 leaves FP32 range: both entry points detect
    it and assemble in FP64 instead."""
    _compare(*_problem(4, True, 5, coef_scale=1e40), precision, RTOL)


def test_no_alloc_unblocked_pattern():
    _compare(*_fan(100, 7), SKG_FP64, RTOL, blocked=False)


def test_no_alloc_empty_mesh():
    X, W = _rule4()
    mesh = sk.MeshTet(np.eye(3, 4), np.zeros((4, 0), dtype=np.int64))
    basis = sk.Basis(mesh, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X, W))
    assert basis.N == 0
    _compare(mesh, basis, X, W, dev.to_device(np.zeros((3, 3, 1)), np.float64), SKG_FP64, RTOL, blocked=False)


def test_no_alloc_rejects_meshes_beyond_its_scratch():
    n = 36  # 36^3 x 6 = 279,936 elements > the fixed maximum
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    assert m.nelements > MAX_ELEMENTS
    basis = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=1),
                     quadrature=(np.full((3, 1), 0.25), np.array([1 / 6])))
    dofs = basis._dev_dofs()
    pat = Pattern(dofs, dofs, m.nelements, 4, 4, basis.N, basis.N)
    out = dev.empty(pat.nnz, np.float64)
    dA = dev.to_device(np.ones((3, 3, m.nelements)), np.float64)
    status = _assemble("skg_h1_assemble_affine_noalloc", pat, m, basis, basis.X, basis.W, dA, SKG_FP64, out)
    assert status != 0
    assert "at most 262144 elements" in load().skg_last_error().decode()
