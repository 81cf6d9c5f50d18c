"""CUDA-graph capture of the FP64 assembly: replays after in-place updates of
the captured inputs give exactly what a fresh assembly gives."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
sk = pytest.importorskip("skfemntv_gb300")

X1 = np.array([[.25], [.25], [.25]])
W1 = np.array([1 / 6])


def test_p2_tensor_capture_replays_new_coefficients():
    from skfemntv_gb300.assembly import NativeTensorForm

    g = load_golden("p2_aniso")
    axis = np.linspace(0.0, 1.0, 13)
    m2 = sk.MeshTet2.from_mesh(sk.MeshTet.init_tensor(axis, axis, axis))
    b = sk.Basis(m2, sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(g["X"], g["W"]))
    E = m2.nelements
    rng = np.random.default_rng(11)
    M = rng.standard_normal((E, 3, 3))
    A = np.ascontiguousarray(np.moveaxis(M @ np.swapaxes(M, 1, 2) + 3.0 * np.eye(3), (1, 2), (0, 1)))
    dA = torch.as_tensor(A, device="cuda")
    form = NativeTensorForm(b)
    graph = form.capture(dA)
    nnz = form.pattern.nnz
    first = graph.replay()[:nnz].clone()
    fresh = form.assemble_device(None, tensor_device=dA)[:nnz].clone()
    assert torch.equal(first, fresh)
    dA.mul_(2.0)  # scaling by two is exact: the replay must give exactly twice the values
    torch.cuda.synchronize()
    second = graph.replay()[:nnz].clone()
    assert torch.equal(second, 2.0 * first)
    M2 = rng.standard_normal((E, 3, 3))
    A2 = np.moveaxis(M2 @ np.swapaxes(M2, 1, 2) + np.eye(3), (1, 2), (0, 1))
    dA.copy_(torch.as_tensor(A2))
    third = graph.replay()[:nnz].clone()
    assert torch.equal(third, form.assemble_device(None, tensor_device=dA)[:nnz])


def test_p1_gradient_capture_replays_new_kappa():
    axis = np.linspace(0.0, 1.0, 17)
    b = sk.Basis(sk.MeshTet.init_tensor(axis, axis, axis), sk.ElementVector(sk.ElementTetP1(), dim=1),
                 quadrature=(X1, W1))
    form = sk.NativeBilinearForm(b)
    kappa = torch.as_tensor(np.exp(np.random.default_rng(2).standard_normal(b.mesh.nelements)), device="cuda")
    graph = form.capture_gradient(kappa)
    nnz = form.pattern.nnz
    kappa.copy_(torch.as_tensor(np.exp(np.random.default_rng(3).standard_normal(b.mesh.nelements))))
    replayed = graph.replay()[:nnz].clone()
    K = sk.asm(sk.BilinearForm(lambda u, v, w: w.kappa * sk.ddot(sk.grad(u), sk.grad(v))), b,
               kappa=kappa.cpu().numpy()[:, None])
    assert np.array_equal(replayed.cpu().numpy(), K.data)
    with pytest.raises(TypeError):
        form.capture_gradient(kappa.float())
