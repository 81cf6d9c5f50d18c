"""Generate the golden fixtures in this folder by running the reference package.

Run in a container that has the reference checkout and its compiled extension
(``oracle/build_ref.sh``)::

    python tests/golden/make_golden.py

Every fixture holds the seeded inputs and the reference's outputs for one
small case shaped like one of the benchmark configurations (P1 Laplace, P2
anisotropic diffusion on a jittered cube, Nedelec N1 Maxwell on a relabelled
cube, vector-P1 elasticity / neo-Hookean pieces, linear forms, geometry and
edge topology).  The fixtures are what pins the CPU oracle and the GPU path.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import reference_loader  # noqa: E402


def jitter(p, h, amp, rng):
    """Move interior vertices by U(-amp*h, amp*h)^3 (boundary vertices stay)."""
    p = p.copy()
    interior = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, interior] += rng.uniform(-amp * h, amp * h, size=(3, int(interior.sum())))
    return p


def spd_tensors(E, rng):
    """A = Q diag(exp(N(0, 0.5^2))) Q^T with Q a sign-fixed QR of a Gaussian."""
    G = rng.standard_normal((E, 3, 3))
    Q, R = np.linalg.qr(G)
    Q = Q * np.sign(np.diagonal(R, axis1=1, axis2=2))[:, None, :]
    lam = np.exp(rng.normal(0.0, 0.5, size=(E, 3)))
    return np.einsum("eij,ej,ekj->eik", Q, lam, Q)


def csr_parts(K):
    K = K.tocsr()
    return dict(indptr=np.asarray(K.indptr, np.int64), indices=np.asarray(K.indices, np.int64),
                data=np.asarray(K.data, np.float64), shape=np.asarray(K.shape, np.int64))


def main():
    sk = reference_loader.load()
    from skfemntv.forms import ddot, dot, grad, mul  # type: ignore
    out = {}

    # --- P1 Laplace, 1-point rule, coefficient 1 and a per-element kappa ---
    m = sk.MeshTet.init_tensor(*(np.linspace(0, 1, 5),) * 3)
    X1, W1 = np.array([[.25], [.25], [.25]]), np.array([1 / 6])
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X1, W1))

    @sk.BilinearForm
    def lap(u, v, w):
        return ddot(grad(u), grad(v))

    @sk.BilinearForm
    def klap(u, v, w):
        return w.kappa * ddot(grad(u), grad(v))

    rng = np.random.default_rng(np.random.SeedSequence(1))
    kappa = np.exp(rng.normal(0, 1, size=m.nelements))
    K = sk.asm(lap, b)
    Kk = sk.asm(klap, b, kappa=kappa[:, None])
    out["p1_laplace"] = dict(p=m.p, t=m.t, X=X1, W=W1, kappa=kappa, **csr_parts(K),
                             kdata=np.asarray(Kk.data).copy())

    # --- P1 default 4-point rule: mass + stiffness with per-(E,Q) coefficients ---
    b4 = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=1))

    @sk.BilinearForm
    def helm(u, v, w):
        return w.c * ddot(grad(u), grad(v)) + w.s * dot(u, v)

    cq = np.exp(rng.normal(0, 0.3, size=b4.dx.shape))
    sq = rng.uniform(0.5, 2.0, size=b4.dx.shape)
    K4 = sk.asm(helm, b4, c=cq, s=sq)
    out["p1_helmholtz"] = dict(p=m.p, t=m.t, X=b4.X, W=b4.W, c=cq, s=sq, **csr_parts(K4),
                               dx=b4.dx, grads=b4.tabulated_gradients)

    # --- P2 anisotropic diffusion, 3^3 x 6 jittered cube, 4-point rule ---
    n = 3
    m0 = sk.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    rng = np.random.default_rng(np.random.SeedSequence(2))
    pj = jitter(m0.p, 1.0 / n, 0.2, rng)
    mj = sk.MeshTet(pj, m0.t)
    m2 = sk.MeshTet2.from_mesh(mj)
    X4, W4 = b4.X, b4.W
    b2 = sk.Basis(m2, sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(X4, W4))
    A = spd_tensors(m2.nelements, rng)  # (E,3,3)
    Apub = np.broadcast_to(np.moveaxis(A, (1, 2), (0, 1))[:, :, :, None], (3, 3, m2.nelements, len(W4)))

    @sk.BilinearForm
    def aniso(u, v, w):
        return dot(mul(w.A, grad(u)), grad(v))

    K2 = sk.asm(aniso, b2, A=np.ascontiguousarray(Apub))
    out["p2_aniso"] = dict(p0=m0.p, pj=pj, t0=m0.t, p=m2.p, t=m2.t, X=X4, W=W4, A=A,
                           **csr_parts(K2), dx=b2.dx, grads=b2.tabulated_gradients,
                           det=b2._geometry_determinants, cond=b2._geometry_condition_numbers,
                           xq=b2.global_coordinates)

    # nonsymmetric tensor variant (the reference keeps nonsymmetric A)
    Ans = A + 0.3 * rng.standard_normal(A.shape)
    Ans_pub = np.broadcast_to(np.moveaxis(Ans, (1, 2), (0, 1))[:, :, :, None], Apub.shape)
    K2n = sk.asm(aniso, b2, A=np.ascontiguousarray(Ans_pub))
    out["p2_aniso"]["Ans"] = Ans
    out["p2_aniso"]["ns_data"] = np.asarray(K2n.data).copy()

    # --- P2 Laplace with the default 11-point rule (negative weight) ---
    b2d = sk.Basis(m2, sk.ElementVector(sk.ElementTetP2(), dim=1))
    K2d = sk.asm(lap, b2d)
    out["p2_laplace_default"] = dict(p=m2.p, t=m2.t, X=b2d.X, W=b2d.W, **csr_parts(K2d))

    # --- the Duffy product rules of the N1 basis, orders 1 to 8 ---
    n1_rules = {}
    for order in range(1, 9):
        bo = sk.AffineTetN1Basis(sk.MeshTet(), intorder=order)
        n1_rules[f"X{order}"], n1_rules[f"W{order}"] = bo.X, bo.W
    out["n1_rules"] = n1_rules

    # --- the basis rules above order 4 (collapsed Gauss-Legendre), and P2 Laplace with order 6 ---
    rules = {}
    for order in (5, 6, 7, 8):
        bo = sk.Basis(sk.MeshTet(), sk.ElementVector(sk.ElementTetP1(), dim=1), intorder=order)
        rules[f"X{order}"], rules[f"W{order}"] = bo.X, bo.W
    b6 = sk.Basis(m2, sk.ElementVector(sk.ElementTetP2(), dim=1), intorder=6)
    out["simplex_rules"] = dict(p=m2.p, t=m2.t, **rules, **csr_parts(sk.asm(lap, b6)))

    # --- curved (isoparametric) P2: the same mesh with its edge nodes moved off the edges'
    #     midpoints (own seed), 4-point rule: geometry, anisotropic diffusion and Laplace ---
    rng_c = np.random.default_rng(np.random.SeedSequence(41))
    pc = m2.p.copy()
    edge_nodes = np.unique(m2.t[4:])
    pc[:, edge_nodes] += 0.02 * rng_c.uniform(-1.0, 1.0, (3, len(edge_nodes)))
    bc = sk.Basis(sk.MeshTet2(pc, m2.t), sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(X4, W4))
    Kc = sk.asm(aniso, bc, A=np.ascontiguousarray(Apub))
    Kcl = sk.asm(lap, bc)
    lap_parts = {f"lap_{k}": v for k, v in csr_parts(Kcl).items()}
    out["p2_curved"] = dict(p=pc, t=m2.t, X=X4, W=W4, A=A, **csr_parts(Kc), **lap_parts, dx=bc.dx,
                            grads=bc.tabulated_gradients, det=bc._geometry_determinants, xq=bc.global_coordinates)

    # --- Nedelec N1 Maxwell, relabelled 3^3 x 6 cube, 27-point Duffy rule ---
    rng = np.random.default_rng(np.random.SeedSequence(3))
    perm = rng.permutation(m0.p.shape[1])
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    p_r = m0.p[:, inv]
    t_r = perm[m0.t]
    mr = sk.MeshTet(p_r, t_r)
    nb = sk.AffineTetN1Basis(mr)
    mu = np.exp(rng.normal(0, 0.3, size=mr.nelements))
    asmb = sk.TetN1Assembler(nb)
    Kn = asmb.assemble_maxwell(mass_coefficient=1.0, curl_coefficient=(1.0 / mu)[:, None])
    topo = nb.dof_map.topology
    out["n1_maxwell"] = dict(p=p_r, t=t_r, mu=mu, X=nb.X, W=nb.W, **csr_parts(Kn),
                             edges=topo.edges, element_edges=topo.element_edges,
                             signs=topo.element_edge_signs, detJ=nb.detJ)

    # --- Nedelec N1 vector load f . phi on the same mesh (own seed) ---
    rng_l = np.random.default_rng(np.random.SeedSequence(31))
    la = sk.TetN1LinearAssembler(nb)
    fq = rng_l.standard_normal((3,) + nb.dx.shape)
    load_arr = la.assemble_vector_load(fq).copy()
    load_fun = la.assemble_vector_load(
        lambda x: np.stack([np.sin(3.0 * x[0]), x[1] * x[2], np.cos(2.0 * x[2]) - x[0]])).copy()
    out["n1_load"] = dict(p=p_r, t=t_r, f=fq, load=load_arr, load_callable=load_fun, xq=nb.global_coordinates)

    # --- Nedelec N1 basis on the same mesh, 3rd-order rule: element matrices, a seeded edge
    #     field evaluated with its curl, edge-moment interpolation of a smooth field ---
    nb3 = sk.AffineTetN1Basis(mr, intorder=3)
    u_edges = np.random.default_rng(np.random.SeedSequence(37)).standard_normal(nb3.N)
    moments = nb3.interpolate_edge_moments(
        lambda x: np.stack([np.sin(3.0 * x[0]) + x[1], x[0] * x[2], np.cos(2.0 * x[2]) - x[0] * x[1]]),
        quadrature_order=4)
    out["n1_basis"] = dict(p=p_r, t=t_r, X=nb3.X, W=nb3.W, mass=nb3.element_mass_matrices(),
                           curl_curl=nb3.element_curl_curl_matrices(), u=u_edges, values=nb3.evaluate(u_edges),
                           curls=nb3.evaluate_curl(u_edges), moments=moments)

    # --- cross-basis assembly: P2 vector test x P1 scalar trial (Stokes coupling),
    #     P2 x P1 scalar mass, and a full gradient tensor on vector P1 ---
    rng_c = np.random.default_rng(np.random.SeedSequence(41))
    mc = sk.MeshTet.init_tensor(*(np.linspace(0, 1, 3),) * 3)
    mc2 = sk.MeshTet2.from_mesh(mc)
    from skfemntv.forms import div as fdiv  # type: ignore
    bv2 = sk.Basis(mc2, sk.ElementVector(sk.ElementTetP2(), dim=3), quadrature=(X4, W4))
    bs1 = sk.Basis(mc2, sk.ElementVector(sk.ElementTetP1(), dim=1), quadrature=(X4, W4))
    bs2 = sk.Basis(mc2, sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(X4, W4))

    @sk.BilinearForm
    def coupling(u, v, w):
        return fdiv(v) * u

    @sk.BilinearForm
    def cmass(u, v, w):
        return w.c * dot(u, v)

    Kb = sk.asm(coupling, bs1, bv2)          # trial P1 scalar, test P2 vector
    cc = rng_c.uniform(0.5, 2.0, size=bs2.dx.shape)
    Km = sk.asm(cmass, bs1, bs2, c=cc)       # trial P1 scalar, test P2 scalar
    bvp1 = sk.Basis(mc, sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(X4, W4))
    T6 = rng_c.standard_normal(bvp1.dx.shape + (3, 3, 3, 3))
    Kt = sk.NativeCrossBilinearForm(bvp1, bvp1).assemble_tensor("gradient", "gradient", T6)
    Tv = rng_c.standard_normal(bvp1.dx.shape + (3, 3))
    Kv = sk.NativeCrossBilinearForm(bvp1, bvp1).assemble_tensor("value", "value", Tv)
    out["cross"] = dict(p0=mc.p, t0=mc.t, p2=mc2.p, t2=mc2.t, X=X4, W=W4, c=cc, T6=T6, Tv=Tv,
                        **{f"b_{k}": v for k, v in csr_parts(Kb).items()},
                        **{f"m_{k}": v for k, v in csr_parts(Km).items()},
                        **{f"t_{k}": v for k, v in csr_parts(Kt).items()},
                        **{f"v_{k}": v for k, v in csr_parts(Kv).items()})

    # --- vector P1 elasticity terms: symmetric gradient + divergence + mass ---
    mv = sk.MeshTet.init_tensor(*(np.linspace(0, 1, 4),) * 3)
    bv = sk.Basis(mv, sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(X1, W1))
    nat = sk.NativeBilinearForm(bv)
    lam_q = np.full(bv.dx.shape, 10.0)
    mu_q = np.full(bv.dx.shape, 1.0)
    Kv = nat.assemble(symmetric_gradient=2 * mu_q, divergence=lam_q, value=0.5 * mu_q)
    out["vp1_elasticity"] = dict(p=mv.p, t=mv.t, X=X1, W=W1, **csr_parts(Kv))

    # --- neo-Hookean residual + tangent (oracle pipeline pieces), vector P1 ---
    rng = np.random.default_rng(np.random.SeedSequence(5))
    u = np.zeros(bv.N)
    xyz = bv.doflocs  # (3, N) repeated per component
    for _ in range(8):
        d = rng.standard_normal(3); d /= np.linalg.norm(d)
        kv = rng.integers(-1, 2, size=3)
        ph = rng.uniform(0, 2 * np.pi)
        comp = np.arange(bv.N) % 3
        u += 0.05 * d[comp] * np.sin(np.pi * (kv @ xyz) + ph)
    dofs3 = bv.element_dofs.T.reshape(mv.nelements, 4, 3)
    Gu = np.einsum("eac,eqaj->eqcj", u[dofs3], bv.tabulated_gradients)
    F = np.eye(3) + Gu
    FiT = np.swapaxes(np.linalg.inv(F), -1, -2)
    lnJ = np.log(np.linalg.det(F))
    mu_, la_ = 1.0, 10.0
    P = mu_ * (F - FiT) + la_ * lnJ[..., None, None] * FiT
    I3 = np.eye(3)
    At = (mu_ * np.einsum("rc,ij->ricj", I3, I3)[None, None]
          + (mu_ - la_ * lnJ)[..., None, None, None, None] * np.einsum("eqrj,eqci->eqricj", FiT, FiT)
          + la_ * np.einsum("eqri,eqcj->eqricj", FiT, FiT))
    res, _ = sk.NativeLinearForm(bv).assemble(gradient=np.ascontiguousarray(P))
    cross = sk.NativeCrossBilinearForm(bv, bv)
    Kt = cross.assemble_tensor("gradient", "gradient", np.ascontiguousarray(At))
    out["nh_vp1"] = dict(p=mv.p, t=mv.t, X=X1, W=W1, u=u, residual=np.asarray(res).copy(),
                         **csr_parts(Kt))

    # --- linear form f.v on P2 with per-(E,Q) f ---
    @sk.LinearForm
    def load(v, w):
        return dot(w.f, v)

    fq = rng.standard_normal(b2.dx.shape)
    rhs = sk.asm(load, b2, f=fq)
    out["p2_load"] = dict(p=m2.p, t=m2.t, X=X4, W=W4, f=fq, rhs=np.asarray(rhs).copy())

    # --- NativeCrossBilinearForm.assemble_kinds on vector P1 (4-point rule): the four value /
    #     gradient pairings with a per-point coefficient of both signs ---
    bkp = sk.Basis(mc, sk.ElementVector(sk.ElementTetP1(), dim=3), quadrature=(X4, W4))
    ck = np.random.default_rng(np.random.SeedSequence(43)).uniform(-1.0, 2.0, bkp.dx.shape)
    kinds = {}
    for row_kind in ("value", "gradient"):
        for column_kind in ("value", "gradient"):
            Kk = sk.NativeCrossBilinearForm(bkp, bkp).assemble_kinds(row_kind, column_kind, ck)
            kinds.update({f"{row_kind}_{column_kind}_{k}": v for k, v in csr_parts(Kk).items()})
    out["cross_kinds"] = dict(p=mc.p, t=mc.t, X=X4, W=W4, c=ck, **kinds)

    # --- volume forms from the reference's compatible-forms cases on vector P1 (default rule):
    #     constant, gradient and coordinate loads; mass, elasticity, coordinate and parameter
    #     coefficients ---
    from skfemntv.helpers import div, sym_grad  # type: ignore

    mf = sk.MeshTet.init_tensor(*(np.linspace(0, 1, 3),) * 3)
    bf = sk.Basis(mf, sk.ElementVector(sk.ElementTetP1(), dim=3), intorder=2)

    @sk.LinearForm
    def force_load(v, w):
        return dot(w.force, v)

    @sk.LinearForm
    def tensor_load(v, w):
        return ddot(w.tensor, grad(v))

    @sk.LinearForm
    def coordinate_load(v, w):
        x = w.x
        return dot(np.stack((1.0 + x[0], x[1] ** 2, -0.5 * x[2]), axis=0), v)

    @sk.BilinearForm
    def vmass(u, v, w):
        return dot(u, v)

    @sk.BilinearForm
    def elasticity(u, v, w):
        return 2.0 * 0.7 * ddot(sym_grad(u), sym_grad(v)) + 2.3 * div(u) * div(v)

    @sk.BilinearForm
    def weighted_mass(u, v, w):
        return (1.0 + w.x[0] ** 2) * dot(u, v)

    @sk.BilinearForm
    def scaled_mass(u, v, w):
        return w.scale * (1.0 + w.x[0]) * dot(u, v)

    @sk.BilinearForm
    def reaction_diffusion(u, v, w):
        return (w.reaction * (1.0 + w.x[0] ** 2) * dot(u, v)
                + w.diffusivity * np.exp(-w.x[1]) * ddot(grad(u), grad(v)))

    tensor = np.arange(9, dtype=float).reshape(3, 3, 1, 1) / 10
    Kf = sk.asm(vmass, bf)
    out["forms_vp1"] = dict(
        p=mf.p, t=mf.t, X=bf.X, W=bf.W, force=np.array([1.2, -0.7, 2.1]), tensor=tensor,
        r_force=np.asarray(sk.asm(force_load, bf, force=np.array([1.2, -0.7, 2.1])[:, None, None])).copy(),
        r_tensor=np.asarray(sk.asm(tensor_load, bf, tensor=tensor)).copy(),
        r_coordinate=np.asarray(sk.asm(coordinate_load, bf)).copy(), **csr_parts(Kf),
        elasticity=np.asarray(sk.asm(elasticity, bf).data).copy(),
        weighted_mass=np.asarray(sk.asm(weighted_mass, bf).data).copy(),
        scaled_mass=np.asarray(sk.asm(scaled_mass, bf, scale=1.8).data).copy(),
        reaction_diffusion=np.asarray(sk.asm(reaction_diffusion, bf, reaction=1.3, diffusivity=0.4).data).copy())

    # --- first-axis coefficient components (scalar P1, default rule) beside a tensor term, and a
    #     component of a linear-form coefficient ---
    mk = sk.MeshTet.init_tensor(np.linspace(0, 1, 5), np.linspace(0, 1, 4), np.linspace(0, 1, 3))
    bk = sk.Basis(mk, sk.ElementVector(sk.ElementTetP1(), dim=1))
    xk = np.moveaxis(bk.global_coordinates, -1, 0)
    material = np.stack((0.7 + 0.2 * xk[0], 1.1 + 0.3 * xk[1]))
    diffusion = np.array([[1.4, 0.2, 0.0], [-0.1, 0.8, 0.1], [0.0, 0.3, 1.2]])
    loads = np.stack((np.full(xk[0].shape, 0.5), 1.0 + xk[0]))

    @sk.BilinearForm
    def components(u, v, w):
        return (w.material[0] * dot(u, v) + w.material[1] * ddot(grad(u), grad(v))
                + dot(mul(w.diffusion, grad(u)), grad(v)))

    @sk.LinearForm
    def component_load(v, w):
        return dot(w.loads[1], v)

    Kk = sk.asm(components, bk, material=material, diffusion=diffusion)
    out["components_p1"] = dict(p=mk.p, t=mk.t, X=bk.X, W=bk.W, material=material, diffusion=diffusion,
                                loads=loads, **csr_parts(Kk),
                                r=np.asarray(sk.asm(component_load, bk, loads=loads)).copy())

    # --- anisotropic forms on the P2 mesh, 4-point rule: a constant (3, 3) tensor, a nonsymmetric
    #     constant tensor with an isotropic mass term, and a scalar coefficient with a unit axis ---
    @sk.BilinearForm
    def aniso_mass(u, v, w):
        return dot(mul(w.A, grad(u)), grad(v)) + 0.25 * dot(u, v)

    @sk.BilinearForm
    def kmass(u, v, w):
        return w.k * dot(u, v)

    Ac = np.array([[2.0, 0.4, 0.1], [0.4, 0.8, -0.2], [0.1, -0.2, 1.3]])
    An = np.array([[1.4, 0.2, 0.0], [-0.1, 0.7, 0.3], [0.05, 0.0, 1.1]])
    E2, Q2 = b2.dx.shape
    kq = 1.0 + np.arange(E2 * Q2, dtype=float).reshape(E2, Q2) / (E2 * Q2)
    Kac = sk.asm(aniso, b2, A=Ac)
    Kam = sk.asm(aniso_mass, b2, A=An)
    out["aniso_forms_p2"] = dict(p=m2.p, t=m2.t, X=X4, W=W4, A_const=Ac, A_nonsym=An, k=kq, **csr_parts(Kac),
                                 combined_indptr=np.asarray(Kam.tocsr().indptr, np.int64),
                                 combined_indices=np.asarray(Kam.tocsr().indices, np.int64),
                                 combined=np.asarray(Kam.tocsr().data).copy(),
                                 kmass=np.asarray(sk.asm(kmass, b2, k=kq[..., None]).data).copy())

    os.makedirs(HERE, exist_ok=True)
    only = set(sys.argv[1:])  # fixture names to (re)write; all when empty
    for name, arrays in out.items():
        if only and name not in only:
            continue
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
        print(f"{name}: {os.path.getsize(path) / 1024:.1f} KiB")


if __name__ == "__main__":
    main()
