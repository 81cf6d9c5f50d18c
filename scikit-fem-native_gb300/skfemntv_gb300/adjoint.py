"""Differentiable energy J = u^T K(kappa) v of P1 diffusion.

``K(kappa)`` is the matrix ``asm(w.kappa * ddot(grad(u), grad(v)), basis)``
assembles for a scalar P1 basis with one kappa per element.  ``P1Energy``
evaluates J matrix-free on the GPU and exposes it as a
``torch.autograd.Function`` with a hand-written adjoint: dJ/dkappa,
dJ/d(node coordinates), dJ/du and dJ/dv.  When an input requires a gradient
the forward call runs one element pass that forms J and the adjoint
contributions for a unit upstream gradient together (the geometry is
computed once; nothing per element is kept), and the backward call scales
the gathered gradients by the upstream gradient.  (The reference has no
autograd; this is the differentiation layer the GPU backend adds on top of
its assembly path.)
"""
from __future__ import annotations

import numpy as np

from . import _device as dev
from ._native import call
from .assembly import Pattern
from .errors import UnsupportedNativeForm


class P1Energy:
    """J(kappa, x, u, v) = u^T K(kappa, x) v on a scalar P1 basis."""

    def __init__(self, basis):
        if basis._quadratic or basis._comp != 1:
            raise UnsupportedNativeForm("P1Energy needs a scalar P1 basis")
        if basis.mesh.t.shape[0] != 4:
            raise UnsupportedNativeForm("P1Energy needs an affine (4-node) tetrahedral mesh")
        self.basis = basis
        mesh = basis.mesh
        self.E = mesh.nelements
        self.npts = mesh.p.shape[1]
        self.t = mesh._dev("t")                        # (4, E)
        self.dofs = basis._dev_dofs()                  # (E, 4)
        vt = self.t.t().contiguous()                   # (E, 4) vertex ids
        self.vertex_inc = Pattern(vt, None, self.E, 4, 0, self.npts, 0)
        if basis.N == self.npts and np.array_equal(basis.element_dofs, mesh.t):
            self.dof_inc = self.vertex_inc             # DOFs are the vertices: one gather walk
        else:
            self.dof_inc = Pattern(self.dofs, None, self.E, 4, 0, basis.N, 0)
        self.wsum = float(np.sum(basis.W))

    def __call__(self, kappa, coords, u, v):
        """kappa (E,), coords (3, npts), u, v (N,): float64 CUDA tensors."""
        return _EnergyFn.apply(kappa, coords, u, v, self)

    # raw entry points (no autograd)
    def energy(self, kappa, coords, u, v):
        import torch

        out = torch.empty(1, dtype=torch.float64, device=coords.device)
        call("skg_p1_energy", dev.ptr(coords), self.npts, dev.ptr(self.t), self.E, dev.ptr(self.dofs),
             dev.ptr(kappa), dev.ptr(u), dev.ptr(v), self.wsum, dev.ptr(out), dev.stream_ptr())
        return out[0]

    def energy_and_gradients(self, kappa, coords, u, v, need=(True, True, True, True)):
        """J and the gradients of J in one element pass (outputs not needed are None)."""
        import torch

        f64 = dict(dtype=torch.float64, device=coords.device)
        out = torch.empty(1, **f64)
        gk = torch.empty(self.E, **f64) if need[0] else None
        gp = torch.empty((3, self.npts), **f64) if need[1] else None
        gu = torch.empty(u.shape[0], **f64) if need[2] else None
        gv = torch.empty(v.shape[0], **f64) if need[3] else None
        call("skg_p1_energy_value_and_grad", self.vertex_inc.h, self.dof_inc.h, dev.ptr(coords), self.npts,
             dev.ptr(self.t), self.E, dev.ptr(self.dofs), dev.ptr(kappa), dev.ptr(u), dev.ptr(v), self.wsum, 1.0,
             dev.ptr(out), dev.ptr(gk), dev.ptr(gp), dev.ptr(gu), dev.ptr(gv), dev.stream_ptr())
        return out[0], gk, gp, gu, gv

    def gradients(self, kappa, coords, u, v, need=(True, True, True, True)):
        import torch

        f64 = dict(dtype=torch.float64, device=coords.device)
        gk = torch.empty(self.E, **f64) if need[0] else None
        gp = torch.empty((3, self.npts), **f64) if need[1] else None
        gu = torch.empty(u.shape[0], **f64) if need[2] else None
        gv = torch.empty(v.shape[0], **f64) if need[3] else None
        call("skg_p1_energy_grad", self.vertex_inc.h, self.dof_inc.h, dev.ptr(coords), self.npts, dev.ptr(self.t),
             self.E, dev.ptr(self.dofs), dev.ptr(kappa), dev.ptr(u), dev.ptr(v), self.wsum, 1.0, dev.ptr(gk),
             dev.ptr(gp), dev.ptr(gu), dev.ptr(gv), dev.stream_ptr())
        return gk, gp, gu, gv


def _check(t, shape, name):
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64:
        raise TypeError(f"{name} must be a float64 CUDA tensor")
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)}")
    return t.contiguous()


try:
    import torch

    class _EnergyFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, kappa, coords, u, v, op):
            kappa = _check(kappa, (op.E,), "kappa")
            coords = _check(coords, (3, op.npts), "coords")
            u = _check(u, (op.basis.N,), "u")
            v = _check(v, (op.basis.N,), "v")
            need = tuple(ctx.needs_input_grad[:4])
            if not any(need):
                return op.energy(kappa, coords, u, v)
            # J and the unit-upstream gradients in one element pass
            J, *grads = op.energy_and_gradients(kappa, coords, u, v, need=need)
            ctx.unit_grads = grads
            return J

        @staticmethod
        def backward(ctx, grad):
            gk, gp, gu, gv = ctx.unit_grads
            del ctx.unit_grads
            scale = lambda g: None if g is None else g * grad  # noqa: E731
            return scale(gk), scale(gp), scale(gu), scale(gv), None
except ImportError:  # pragma: no cover
    _EnergyFn = None
