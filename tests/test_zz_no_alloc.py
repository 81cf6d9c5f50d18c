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
from skfemntv_gb300._native import SKG_FP64, SKG_FP64_EMULATED, load  # noqa: E402
from skfemntv_gb300.assembly import Pattern  # noqa: E402

RTOL = 1e-12
MAX_ELEMENTS = 262144


def _problem(n, quadratic, seed):
    rng = np.random.default_rng(seed)
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    p = m.p.copy()
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
    mesh = sk.MeshTet(p, m.t)
    if quadratic:
        mesh = sk.MeshTet2.from_mesh(mesh)
    a, b = 0.5854101966249685, 0.1381966011250105
    X = np.array([[a, b, b, b], [b, a, b, b], [b, b, a, b]])
    W = np.full(4, 1.0 / 24.0)
    elem = sk.ElementTetP2() if quadratic else sk.ElementTetP1()
    basis = sk.Basis(mesh, sk.ElementVector(elem, dim=1), quadrature=(X, W))
    E = mesh.nelements
    A = rng.standard_normal((3, 3, E))
    A = np.ascontiguousarray(np.einsum("ije,kje->ike", A, A) + 3.0 * np.eye(3)[:, :, None])
    return mesh, basis, X, W, dev.to_device(A, np.float64)


def _assemble(name, pat, mesh, basis, X, W, dA, precision, out):
    lib = load()
    L = basis._nodes
    args = [pat.h, dev.ptr(mesh._dev("p")), mesh.p.shape[1], dev.ptr(mesh._dev("t")), L, mesh.nelements]
    if name == "skg_h1_assemble_affine":
        args.append(dev.ptr(basis._dev_dofs()))
    args += [len(W), dev.hptr(X), dev.hptr(W), 2, dev.ptr(dA), precision, dev.ptr(out), dev.stream_ptr()]
    status = getattr(lib, name)(*args)
    torch.cuda.synchronize()
    return status


@pytest.mark.parametrize("quadratic,precision", [(False, SKG_FP64), (True, SKG_FP64), (True, SKG_FP64_EMULATED)])
def test_no_alloc_matches_allocating_entry_point(quadratic, precision):
    mesh, basis, X, W, dA = _problem(5 if quadratic else 8, quadratic, 3)
    L = basis._nodes
    dofs = basis._dev_dofs()
    pat = Pattern(dofs, dofs, mesh.nelements, L, L, basis.N, basis.N)
    ref = dev.empty(pat.nnz, np.float64)
    got = dev.empty(pat.nnz, np.float64)
    assert _assemble("skg_h1_assemble_affine", pat, mesh, basis, X, W, dA, precision, ref) == 0
    for call in range(2):  # two calls in a row share the static scratch array
        got.fill_(float("nan"))
        assert _assemble("skg_h1_assemble_affine_noalloc", pat, mesh, basis, X, W, dA, precision, got) == 0
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        assert np.all(np.isfinite(g)), call
        assert np.max(np.abs(g - r)) <= RTOL * np.max(np.abs(r)), call


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
