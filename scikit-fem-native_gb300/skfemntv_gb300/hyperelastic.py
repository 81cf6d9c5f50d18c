"""Neo-Hookean residual / tangent assembly and its learned energy closure.

``NeoHookean`` assembles, on a vector P1 basis, the residual and tangent of
the neo-Hookean law the reference keeps as scikit-fem forms
(benchmarks/skfem_neo_hookean.py:8-52), which the reference assembles with
NativeLinearForm and NativeCrossBilinearForm.assemble_tensor.  FP64
throughout (plain law).

``EnergySurrogate`` is the learned part: an MLP 3 -> 64 -> 64 -> 1 (tanh, with
a linear input -> output skip) on the invariants (I1, I2, J) predicting the
strain energy, trained on the GPU by the library's own forward / backward
kernels, on samples F = I + G (G_ij ~ N(0, sigma^2)) that the plain law
labels: Adam on mini-batches, then L-BFGS on a fixed sample window (each
loss / gradient evaluation on the device).  With a surrogate,
``NeoHookean.assemble`` derives stress and tangent from the network's first
and second derivatives, and falls back to the plain law per element outside
the trained invariant range or when the element's stress disagrees with the
plain law (``tol``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _device as dev
from ._native import call, load
from .assembly import Pattern, _MatrixTarget
from .errors import UnsupportedNativeForm


class EnergySurrogate:
    """MLP strain-energy surrogate (float32 parameters on the device)."""

    HIDDEN = 64

    def __init__(self, params, box, mu, lmbda):
        self.params = params  # torch float32 CUDA tensor (skg_mlp_param_count())
        self.box = box        # torch float32 CUDA tensor (6,)
        self.mu, self.lmbda = float(mu), float(lmbda)
        self.history = []

    @staticmethod
    def n_params():
        return int(load().skg_mlp_param_count())

    @classmethod
    def initial(cls, mu, lmbda, f_mean, f_std, y_scale, y_shift, box, skip=(0.0, 0.0, 0.0), seed=0):
        """Glorot-uniform weights, zero biases; ``skip`` starts the linear term."""
        import torch

        H = cls.HIDDEN
        rng = np.random.default_rng(seed)
        w1 = rng.uniform(-1, 1, (H, 3)) * np.sqrt(6.0 / (3 + H))
        w2 = rng.uniform(-1, 1, (H, H)) * np.sqrt(6.0 / (2 * H))
        w3 = rng.uniform(-1, 1, H) * np.sqrt(6.0 / (H + 1))
        p = np.concatenate([w1.ravel(), np.zeros(H), w2.ravel(), np.zeros(H), w3, [0.0], np.asarray(skip, float),
                            f_mean, f_std, [y_scale, y_shift, 0.0]]).astype(np.float32)
        assert p.size == cls.n_params()
        return cls(torch.as_tensor(p, device="cuda"), torch.as_tensor(np.asarray(box, np.float32), device="cuda"),
                   mu, lmbda)

    @classmethod
    def train(cls, mu=1.0, lmbda=10.0, n_samples=2_000_000, sigma=0.1, steps=3000, batch=16384, lr=3e-3,
              lr_min=1e-5, beta=4.0, refine_iters=12000, refine_samples=524288, history=50, seed=0):
        """Generate plain-law samples and fit the network on the GPU.

        ``steps`` Adam steps on mini-batches of ``batch`` samples, then up to
        ``refine_iters`` L-BFGS iterations on ``refine_samples`` fixed samples.
        ``history`` records (stage, iteration, loss)."""
        import torch

        feats = torch.empty((n_samples, 3), dtype=torch.float32, device="cuda")
        tgts = torch.empty((n_samples, 4), dtype=torch.float32, device="cuda")
        call("skg_mlp_dataset", n_samples, seed, sigma, mu, lmbda, dev.ptr(feats), dev.ptr(tgts), dev.stream_ptr())
        f_mean = feats.mean(0).double().cpu().numpy()
        f_std = feats.std(0).double().cpu().numpy()
        y_shift = float(tgts[:, 0].mean())
        y_scale = float(tgts[:, 0].std())
        box = np.concatenate([feats.min(0).values.double().cpu().numpy(), feats.max(0).values.double().cpu().numpy()])
        # the skip starts at the mean normalised feature gradient (the linear part of W)
        skip = (tgts[:, 1:].double().mean(0).cpu().numpy() * f_std / y_scale)
        model = cls.initial(mu, lmbda, f_mean, f_std, y_scale, y_shift, box, skip=skip, seed=seed)
        g = torch.Generator().manual_seed(seed)
        perm = torch.randperm(n_samples, generator=g).to(device="cuda", dtype=torch.int64)
        m = torch.zeros(model.n_params(), dtype=torch.float32, device="cuda")
        v = torch.zeros_like(m)
        loss = ctypes.c_float()
        chunk = 250
        done = 0
        while done < steps:
            k = min(chunk, steps - done)
            call("skg_mlp_train", dev.ptr(model.params), dev.ptr(feats), dev.ptr(tgts), n_samples, dev.ptr(perm), k,
                 batch, ctypes.c_float(lr), ctypes.c_float(lr_min), ctypes.c_float(beta), dev.ptr(m), dev.ptr(v), done,
                 ctypes.byref(loss), dev.stream_ptr())
            done += k
            model.history.append(("adam", done, float(loss.value)))
        if refine_iters > 0:
            floss = ctypes.c_double()
            count = min(refine_samples, n_samples)
            call("skg_mlp_refine", dev.ptr(model.params), dev.ptr(feats), dev.ptr(tgts), n_samples, dev.ptr(perm), 0,
                 count, refine_iters, history, ctypes.c_float(beta), ctypes.byref(floss), dev.stream_ptr())
            model.history.append(("lbfgs", refine_iters, float(floss.value)))
        model.training_set = (feats, tgts, perm)
        return model

    def evaluate(self, x):
        """psi, grad psi (3), Hessian (9) at normalised inputs x (n, 3) float32 CUDA."""
        import torch

        out = torch.empty((x.shape[0], 13), dtype=torch.float32, device="cuda")
        call("skg_mlp_eval", dev.ptr(self.params), dev.ptr(x.contiguous()), x.shape[0], dev.ptr(out),
             dev.stream_ptr())
        return out

    def loss_and_grad(self, feats, tgts, perm, offset, batch, beta=1.0):
        import torch

        grad = torch.empty(self.n_params(), dtype=torch.float32, device="cuda")
        loss = torch.empty(1, dtype=torch.float32, device="cuda")
        call("skg_mlp_loss_grad", dev.ptr(self.params), dev.ptr(feats), dev.ptr(tgts), feats.shape[0], dev.ptr(perm),
             offset, batch, ctypes.c_float(beta), dev.ptr(grad), dev.ptr(loss), dev.stream_ptr())
        return float(loss.item()), grad


class NeoHookean:
    """Neo-Hookean residual and tangent on a vector P1 basis."""

    def __init__(self, basis, mu=1.0, lmbda=10.0):
        if basis._quadratic or basis._comp != 3 or basis.mesh.t.shape[0] != 4:
            raise UnsupportedNativeForm("neo-Hookean assembly needs a vector P1 basis on a 4-node tet mesh")
        self.basis = basis
        self.mu, self.lmbda = float(mu), float(lmbda)
        E = basis.mesh.nelements
        dofs = basis._dev_dofs()
        self.pattern = Pattern(dofs, dofs, E, 12, 12, basis.N, basis.N)
        self.target = _MatrixTarget(self.pattern, (basis.N, basis.N))
        self.d_res = dev.empty(max(1, basis.N), np.float64)
        self.wsum = float(np.sum(basis.W))
        self.last_fallback = 0
        self._res_pinned = self._res_host = None

    def _launch(self, u_ptr, surrogate, tol, res_ptr, val_ptr, count_fallback, host=None):
        """host: (residual, values) page-locked host pointers that also receive
        the results (copied chunk by chunk while later chunks run)."""
        b = self.basis
        mesh = (self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1], dev.ptr(b.mesh._dev("t")),
                b.mesh.nelements, u_ptr, self.mu, self.lmbda, self.wsum)
        if surrogate is None:
            self.last_fallback = 0
            if host is None:
                call("skg_nh_assemble", *mesh, res_ptr, val_ptr, dev.stream_ptr())
            else:
                call("skg_nh_assemble_host", *mesh, res_ptr, val_ptr, *host, dev.stream_ptr())
        else:
            fb = ctypes.c_int64(-1)
            net = (dev.ptr(surrogate.params), dev.ptr(surrogate.box), ctypes.c_float(tol), res_ptr, val_ptr)
            count = ctypes.byref(fb) if count_fallback else None
            if host is None:
                call("skg_nh_assemble_surrogate", *mesh, *net, count, dev.stream_ptr())
            else:
                call("skg_nh_assemble_surrogate_host", *mesh, *net, *host, count, dev.stream_ptr())
            self.last_fallback = int(fb.value)

    def assemble_device(self, u, surrogate=None, tol=1e-3, residual=True, tangent=True, count_fallback=True):
        """Residual / tangent into device buffers.  With ``count_fallback`` the
        number of plain-law elements is read back (a host synchronisation)."""
        du = u if hasattr(u, "data_ptr") else dev.to_device(np.asarray(u, dtype=np.float64), np.float64)
        r = self.d_res if residual else None
        k = self.target.d_values if tangent else None
        self._launch(dev.ptr(du), surrogate, tol, dev.ptr(r), dev.ptr(k), count_fallback)
        return r, k

    def assemble(self, u, surrogate=None, tol=1e-3):
        """(residual vector, tangent csr_matrix) at displacement u (N,).  The
        tangent matrix is reused between calls.  A host u is read by the device in
        place when it can (the library copies it to the device first); the
        residual and the CSR values reach page-locked host buffers row chunk by
        row chunk while the later chunks are computed."""
        if hasattr(u, "data_ptr"):
            self.assemble_device(u, surrogate=surrogate, tol=tol)
            K = self.target.download()
            return self.d_res[: self.basis.N].cpu().numpy(), K
        ua = np.ascontiguousarray(np.asarray(u, dtype=np.float64))
        u_ptr = dev.host_readable(ua)
        keep = None
        if u_ptr is None:
            keep = dev.to_device(ua, np.float64)
            u_ptr = dev.ptr(keep)
        if self._res_pinned is None:
            self._res_pinned, self._res_host = dev.pinned_empty(max(1, self.basis.N))
        self._launch(u_ptr, surrogate, tol, dev.ptr(self.d_res), dev.ptr(self.target.d_values), True,
                     host=(ctypes.c_void_p(self._res_pinned.data_ptr()), self.target.pinned_ptr()))
        K = self.target.finish_direct()
        del keep
        return dev.host_copy(self._res_host[: self.basis.N]), K
