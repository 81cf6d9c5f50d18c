"""Adjoint of J = u^T K(kappa) v for P1 diffusion (GPU), checked against the
oracle's assembled matrix, exact directional derivatives through the plain
FP64 assembly, and central finite differences (h = 1e-6)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
sk = pytest.importorskip("skfemntv_gb300")

X1 = np.array([[.25], [.25], [.25]])
W1 = np.array([1 / 6])


def problem(n=4, seed=4):
    rng = np.random.default_rng(np.random.SeedSequence(seed))
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    p = m.p.copy()
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
    mesh = sk.MeshTet(p, m.t)
    basis = sk.Basis(mesh, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X1, W1))
    E = mesh.nelements
    kappa = np.exp(rng.normal(0, 1, E))
    u = rng.standard_normal(basis.N)
    v = rng.standard_normal(basis.N)
    return mesh, basis, kappa, u, v


def oracle_energy(p, t, kappa, u, v):
    ob = O.make_basis(p, t, False, quadrature=(X1, W1))
    data, indptr, indices = O.bilinear_assemble(ob, gradient=kappa[:, None])
    import scipy.sparse as sp

    K = sp.csr_matrix((data, indices, indptr), shape=(ob.N, ob.N))
    return float(u @ (K @ v)), K


def cuda(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def test_energy_and_gradients():
    mesh, basis, kappa, u, v = problem()
    op = sk.P1Energy(basis)
    kt, pt, ut, vt = (cuda(a).requires_grad_(True) for a in (kappa, mesh.p, u, v))
    J = op(kt, pt, ut, vt)
    Jref, K = oracle_energy(mesh.p, mesh.t, kappa, u, v)
    assert abs(J.item() - Jref) <= 1e-12 * abs(Jref)
    J.backward()
    # dJ/du = K v, dJ/dv = K^T u (assembled by the oracle)
    assert np.max(np.abs(ut.grad.cpu().numpy() - K @ v)) <= 1e-12 * np.max(np.abs(K @ v))
    assert np.max(np.abs(vt.grad.cpu().numpy() - K.T @ u)) <= 1e-12 * np.max(np.abs(K.T @ u))
    # dJ/dkappa_e = J(unit kappa on e): exact, through the plain FP64 assembly
    gk = kt.grad.cpu().numpy()
    rng = np.random.default_rng(0)
    for e in rng.choice(mesh.nelements, 20, replace=False):
        ke = np.zeros(mesh.nelements)
        ke[e] = 1.0
        Je, _ = oracle_energy(mesh.p, mesh.t, ke, u, v)
        assert abs(gk[e] - Je) <= 1e-12 * max(abs(Je), 1e-300) + 1e-14 * np.max(np.abs(gk))
    # dJ/dx: central differences (h = 1e-6) through the oracle forward path
    gp = pt.grad.cpu().numpy()
    inner = np.flatnonzero(np.all((mesh.p > 1e-12) & (mesh.p < 1 - 1e-12), axis=0))
    h = 1e-6
    for node in rng.choice(inner, 10, replace=False):
        for i in range(3):
            pp = mesh.p.copy(); pp[i, node] += h
            pm = mesh.p.copy(); pm[i, node] -= h
            fd = (oracle_energy(pp, mesh.t, kappa, u, v)[0] - oracle_energy(pm, mesh.t, kappa, u, v)[0]) / (2 * h)
            assert abs(gp[i, node] - fd) <= 1e-6 * max(1.0, abs(fd)), (node, i, gp[i, node], fd)


def test_gradient_matches_own_fd_and_is_deterministic():
    mesh, basis, kappa, u, v = problem(n=3, seed=9)
    op = sk.P1Energy(basis)
    kt, pt, ut, vt = (cuda(a) for a in (kappa, mesh.p, u, v))
    g1 = op.gradients(kt, pt, ut, vt)
    g2 = op.gradients(kt, pt, ut, vt)
    for a, b in zip(g1, g2):
        assert torch.equal(a, b)
    # directional FD of J along a random kappa direction through our forward
    d = cuda(np.random.default_rng(1).standard_normal(mesh.nelements))
    h = 1e-6
    fd = (op.energy(kt + h * d, pt, ut, vt) - op.energy(kt - h * d, pt, ut, vt)).item() / (2 * h)
    an = float((g1[0] * d).sum())
    assert abs(an - fd) <= 1e-7 * max(1.0, abs(an))


def test_shared_and_separate_incidence_walks_agree():
    """Scalar P1 (DOFs = vertices) gathers all gradients in one walk over the
    vertex incidences; the two-walk path over separate handles gives the same
    bits."""
    from skfemntv_gb300.assembly import Pattern

    mesh, basis, kappa, u, v = problem(n=3, seed=5)
    kt, pt, ut, vt = (cuda(a) for a in (kappa, mesh.p, u, v))
    op = sk.P1Energy(basis)
    assert op.dof_inc is op.vertex_inc
    g1 = op.gradients(kt, pt, ut, vt)
    op.dof_inc = Pattern(op.dofs, None, op.E, 4, 0, basis.N, 0)
    g2 = op.gradients(kt, pt, ut, vt)
    for a, b in zip(g1, g2):
        assert torch.equal(a, b)


def test_fused_value_and_gradients_match_separate_passes():
    """The forward pass of the autograd function (J and unit-upstream gradients in one element pass) gives the
    bits of the separate energy and gradient calls, for every subset of inputs that require a gradient."""
    mesh, basis, kappa, u, v = problem(n=4, seed=6)
    op = sk.P1Energy(basis)
    base = [cuda(a) for a in (kappa, mesh.p, u, v)]
    J0 = op.energy(*base)
    g0 = op.gradients(*base)
    J1, *g1 = op.energy_and_gradients(*base)
    assert torch.equal(J0, J1)
    for a, b in zip(g0, g1):
        assert torch.equal(a, b)
    for need in [(True, False, False, False), (False, True, False, False), (False, False, True, True),
                 (True, True, True, True)]:
        ins = [t.clone().requires_grad_(r) for t, r in zip(base, need)]
        J = op(*ins)
        assert torch.equal(J.detach(), J0)
        (2.5 * J).backward()
        for t, r, g in zip(ins, need, g0):
            if r:
                assert torch.equal(t.grad, g * 2.5)
            else:
                assert t.grad is None
    with torch.no_grad():
        assert torch.equal(op(*[t.clone().requires_grad_(True) for t in base]), J0)


def patch_energy(p, t, patch, kappa, u, v):
    """J restricted to the elements `patch` (every other element's term is
    unchanged by the perturbations below), through the oracle's assembly."""
    sub = np.ascontiguousarray(t[:, patch])
    active = np.unique(sub)  # the oracle compacts to these vertices, in this order
    J, _ = oracle_energy(p, sub, kappa[patch], u[active], v[active])
    return J


def test_fd_gradients_on_the_64_cube():
    """The benchmark's adjoint size, 64^3 x 6 (1,572,864 tets), interior
    vertices jittered: dJ/dkappa on 100 seeded elements and dJ/dx on 100
    seeded interior coordinates against central differences (h = 1e-6).
    J is a sum of element terms, so each difference is taken over the
    elements the perturbed kappa_e or vertex touches (the oracle assembles
    that patch); the other terms cancel exactly."""
    mesh, basis, kappa, u, v = problem(n=64, seed=4)
    assert mesh.nelements == 1572864
    op = sk.P1Energy(basis)
    kt, pt, ut, vt = (cuda(a).requires_grad_(True) for a in (kappa, mesh.p, u, v))
    op(kt, pt, ut, vt).backward()
    gk, gp = kt.grad.cpu().numpy(), pt.grad.cpu().numpy()
    p, t = mesh.p, mesh.t
    h = 1e-6
    rng = np.random.default_rng(np.random.SeedSequence(200))
    worst = 0.0
    for e in rng.choice(mesh.nelements, 100, replace=False):
        kp, km = kappa.copy(), kappa.copy()
        kp[e] += h
        km[e] -= h
        fd = (patch_energy(p, t, [e], kp, u, v) - patch_energy(p, t, [e], km, u, v)) / (2 * h)
        err = abs(gk[e] - fd) / max(abs(fd), 1e-3 * np.max(np.abs(gk)))
        worst = max(worst, err)
        assert err <= 1e-7, (e, gk[e], fd)
    inner = np.flatnonzero(np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0))
    scale = np.max(np.abs(gp[:, inner]))
    for node, i in zip(rng.choice(inner, 100, replace=False), rng.integers(0, 3, 100)):
        patch = np.flatnonzero(np.any(t == node, axis=0))
        pp, pm = p.copy(), p.copy()
        pp[i, node] += h
        pm[i, node] -= h
        fd = (patch_energy(pp, t, patch, kappa, u, v) - patch_energy(pm, t, patch, kappa, u, v)) / (2 * h)
        err = abs(gp[i, node] - fd) / max(abs(fd), 1e-3 * scale)
        worst = max(worst, err)
        assert err <= 1e-6, (node, i, gp[i, node], fd)
    print(f"64^3 adjoint vs central differences: worst relative error {worst:.2e}")
