"""Neo-Hookean residual / tangent (plain law) and the learned energy closure
on the GPU, against the reference's golden outputs and the CPU oracle."""
import numpy as np
import pytest

import oracle as O
from conftest import load_golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
sk = pytest.importorskip("skfemntv_gb300")

X1 = np.array([[.25], [.25], [.25]])
W1 = np.array([1 / 6])


def relerr(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def test_plain_law_matches_reference():
    g = load_golden("nh_vp1")
    b = sk.Basis(sk.MeshTet(g["p"], g["t"]), sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(g["X"], g["W"]))
    nh = sk.NeoHookean(b, 1.0, 10.0)
    r, K = nh.assemble(g["u"])
    assert relerr(r, g["residual"]) < 1e-12
    assert np.array_equal(K.indptr, g["indptr"]) and np.array_equal(K.indices, g["indices"])
    assert relerr(K.data, g["data"]) < 1e-12


def test_network_derivatives_match_cpu_oracle(surrogate):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((257, 3)).astype(np.float32)
    out = surrogate.evaluate(torch.as_tensor(x, device="cuda")).cpu().numpy()
    psi, g, H = O.mlp_eval(surrogate.params.cpu().numpy(), x)
    assert np.max(np.abs(out[:, 0] - psi)) <= 1e-5 * max(1.0, np.max(np.abs(psi)))
    assert np.max(np.abs(out[:, 1:4] - g)) <= 1e-5 * max(1.0, np.max(np.abs(g)))
    assert np.max(np.abs(out[:, 4:].reshape(-1, 3, 3) - H)) <= 1e-4 * max(1.0, np.max(np.abs(H)))


def check_gradient(model, feats, tgts, perm, batch=512, beta=1.0, rtol=2e-3):
    loss, grad = model.loss_and_grad(feats, tgts, perm, 0, batch, beta=beta)
    idx = perm[:batch].cpu().numpy()
    f = feats.cpu().numpy()[idx]
    t = tgts.cpu().numpy()[idx]
    p0 = model.params.cpu().numpy().astype(np.float64)
    assert abs(loss - O.mlp_loss(p0, f, t, beta)) <= 1e-4 * max(loss, 1e-12) + 1e-9
    grad = grad.cpu().numpy()
    n_trainable = O.MLP_N_TRAINABLE
    rng = np.random.default_rng(0)
    picks = np.concatenate([rng.choice(np.arange(0, 256), 6, replace=False),
                            rng.choice(np.arange(256, 256 + 4096), 10, replace=False),
                            rng.choice(np.arange(256 + 4096, n_trainable - 4), 6, replace=False),
                            np.arange(n_trainable - 4, n_trainable)])
    h = 1e-4
    scale = np.max(np.abs(grad[:n_trainable]))
    for k in picks:
        pp = p0.copy(); pp[k] += h
        pm = p0.copy(); pm[k] -= h
        fd = (O.mlp_loss(pp, f, t, beta) - O.mlp_loss(pm, f, t, beta)) / (2 * h)
        assert abs(grad[k] - fd) <= rtol * scale + 1e-3 * abs(fd), (k, grad[k], fd)


def test_training_gradient_matches_cpu_oracle(surrogate):
    feats, tgts, perm = surrogate.training_set
    p = surrogate.params.cpu().numpy()
    norm = p[O.MLP_N_TRAINABLE:]
    fresh = sk.EnergySurrogate.initial(1.0, 10.0, norm[:3], norm[3:6], norm[6], norm[7], surrogate.box.cpu().numpy(),
                                       skip=(0.3, -0.2, 0.1), seed=7)
    check_gradient(fresh, feats, tgts, perm, beta=0.5)   # untrained weights: large gradient
    # trained weights: the gradient is a small sum of cancelling per-sample
    # terms, so FP32 accumulation error is large relative to it
    check_gradient(surrogate, feats, tgts, perm, beta=4.0, rtol=5e-2)


def test_training_converges(surrogate):
    adam = [h for h in surrogate.history if h[0] == "adam"]
    final = surrogate.history[-1]
    assert final[0] == "lbfgs"
    assert final[2] < 0.01 * adam[-1][2]
    assert final[2] < 2e-7


def sine_displacement(basis, seed=5, amplitude=0.05):
    """u = sum of 8 modes amplitude * d_m sin(pi k_m . x + phi_m), seeded unit
    directions d_m, phases phi_m and unit wavevectors k_m = +-e_axis (the
    element deformation gradients then stay inside the spread of the training
    samples G_ij ~ N(0, 0.1^2))."""
    rng = np.random.default_rng(np.random.SeedSequence(seed))
    u = np.zeros(basis.N)
    xyz = basis.doflocs
    comp = np.arange(basis.N) % 3
    for _ in range(8):
        d = rng.standard_normal(3); d /= np.linalg.norm(d)
        kv = np.zeros(3); kv[rng.integers(0, 3)] = rng.choice([-1.0, 1.0])
        ph = rng.uniform(0, 2 * np.pi)
        u += amplitude * d[comp] * np.sin(np.pi * (kv @ xyz) + ph)
    return u


# Max relative error against the FP64 plain law (residual and tangent) that
# the default training recipe must reach.
SURROGATE_RTOL = 1e-4


def test_surrogate_assembly_accuracy_and_fallback(surrogate):
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, 13),) * 3)
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(X1, W1))
    nh = sk.NeoHookean(b, 1.0, 10.0)
    u = sine_displacement(b)
    r0, K0 = nh.assemble(u)
    r0 = r0.copy(); d0 = K0.data.copy()
    assert nh.last_fallback == 0
    r1, K1 = nh.assemble(u, surrogate=surrogate, tol=1e-2)
    assert nh.last_fallback == 0
    er, ek = relerr(r1, r0), relerr(K1.data, d0)
    print(f"surrogate max relative error: residual {er:.3e}, tangent {ek:.3e}")
    assert er < SURROGATE_RTOL and ek < SURROGATE_RTOL
    # every element failing the stress check: the FP64 plain law everywhere
    # (summed in double-float slots on the surrogate path)
    r2, K2 = nh.assemble(u, surrogate=surrogate, tol=-1.0)
    assert nh.last_fallback == m.nelements
    assert relerr(r2, r0) < 1e-13 and relerr(K2.data, d0) < 1e-13
    # larger deformations: elements outside the trained range fall back
    u3 = sine_displacement(b, amplitude=0.2)
    r3, K3 = nh.assemble(u3)
    r3 = r3.copy(); d3 = K3.data.copy()
    r4, K4 = nh.assemble(u3, surrogate=surrogate, tol=1e-2)
    assert 0 < nh.last_fallback < m.nelements
    assert relerr(r4, r3) < 3e-2 and relerr(K4.data, d3) < 5e-2


def test_surrogate_is_faster_than_plain_law(surrogate):
    """What the trained network gains: on a 48^3 x 6 mesh the surrogate
    residual + tangent assembly (tensor-core network, FP32 rows) takes less
    time than the FP64 plain law (itself FP64-pipe bound), at the accuracy
    asserted above."""
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, 49),) * 3)
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(X1, W1))
    nh = sk.NeoHookean(b, 1.0, 10.0)
    du = torch.as_tensor(sine_displacement(b), dtype=torch.float64, device="cuda")

    def best_ms(fn, reps=7):
        for _ in range(2):
            fn()
        times = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return min(times)

    t_plain = best_ms(lambda: nh.assemble_device(du))
    t_sur = best_ms(lambda: nh.assemble_device(du, surrogate=surrogate, tol=1e-2, count_fallback=False))
    nh.assemble_device(du, surrogate=surrogate, tol=1e-2)
    print(f"48^3 plain {t_plain:.3f} ms, surrogate {t_sur:.3f} ms, fallback {nh.last_fallback}")
    assert nh.last_fallback == 0
    assert t_sur < t_plain


@pytest.mark.parametrize("cells", [16, 34])
def test_host_output_matches_device(surrogate, cells):
    """The host-output path (u read from host memory; at 34^3, 5.4 M values,
    element and row passes over row chunks with the results copied chunk by
    chunk) returns exactly the device path's residual and tangent, for the
    plain law, the surrogate and the all-fallback surrogate."""
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, cells + 1),) * 3)
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(X1, W1))
    nh = sk.NeoHookean(b, 1.0, 10.0)
    assert nh.pattern.row_groups
    u = sine_displacement(b)
    du = torch.as_tensor(u, dtype=torch.float64, device="cuda")
    import ctypes
    from skfemntv_gb300 import _device as dev

    res_pinned, res_view = dev.pinned_empty(b.N)
    val_pinned, val_view = dev.pinned_empty(nh.pattern.nnz)
    for kw in ({}, {"surrogate": surrogate, "tol": 1e-2}, {"surrogate": surrogate, "tol": -1.0}):
        r_host, K_host = nh.assemble(u, **kw)
        fb_host = nh.last_fallback
        r_host, d_host = r_host.copy(), K_host.data.copy()
        r_dev, k_dev = nh.assemble_device(du, **kw)
        assert nh.last_fallback == fb_host
        r_dev, k_dev = r_dev[: b.N].cpu().numpy(), k_dev[: nh.pattern.nnz].cpu().numpy()
        assert np.array_equal(r_host.view(np.int64), r_dev.view(np.int64))
        assert np.array_equal(d_host.view(np.int64), k_dev.view(np.int64))
        # the chunked host-output entry points (device staging, copies per row chunk)
        nh._launch(dev.ptr(du), kw.get("surrogate"), kw.get("tol", 1e-3), dev.ptr(nh.d_res),
                   dev.ptr(nh.target.d_values), True,
                   host=(ctypes.c_void_p(res_pinned.data_ptr()), ctypes.c_void_p(val_pinned.data_ptr())))
        torch.cuda.synchronize()
        assert nh.last_fallback == fb_host
        assert np.array_equal(res_view.view(np.int64), r_dev.view(np.int64))
        assert np.array_equal(val_view.view(np.int64), k_dev.view(np.int64))
