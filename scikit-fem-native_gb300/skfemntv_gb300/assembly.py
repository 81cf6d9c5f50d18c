"""GPU assemblers behind ``asm`` (python/skfemntv/bilinear_form.py:13-367,
linear_form.py:17-107, forms.py:276-404).

Ownership follows the reference: the plain bilinear path returns one reused
``csr_matrix`` whose values are overwritten by the next call on the same
(form, basis); the tensor (anisotropic) path returns a fresh copy.  The CSR
pattern is built once per (form, basis) on the device.

Path selection for scalar P1/P2 on affine meshes with coefficients that are
constant over each element's quadrature points: the fused affine kernel
(geometry + contraction + fixed-order CSR sum from coordinates).  Anything
else (vector fields, symmetric-gradient / divergence / mass terms, per-point
coefficients, curved P2 geometry) goes through the tabulated path (device
geometry tabulation, element matrices, the same fixed-order gather).
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass

import numpy as np
from scipy.sparse import csr_matrix

from . import _device as dev
from ._native import SKG_FP64, SKG_FP64_EMULATED, SKG_SPLIT_FP32, call
from .errors import UnsupportedNativeForm
from .preflight import enforce_memory_budget, estimate_bilinear_memory

PRECISIONS = {"fp64": SKG_FP64, "fp64_emulated": SKG_FP64_EMULATED, "split_fp32": SKG_SPLIT_FP32}


def _precision(name):
    try:
        return PRECISIONS[name]
    except KeyError:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}") from None


class Pattern:
    """Device CSR pattern + row incidence lists (skg_pattern handle)."""

    def __init__(self, row_dofs_dev, col_dofs_dev, n_elements, row_local, col_local, n_rows, n_cols):
        h = ctypes.c_void_p()
        call("skg_pattern_create", dev.ptr(row_dofs_dev), dev.ptr(col_dofs_dev), n_elements, row_local,
             col_local, n_rows, n_cols, dev.stream_ptr(), ctypes.byref(h))
        self.h = h
        nnz = ctypes.c_int64()
        call("skg_pattern_info", h, ctypes.byref(nnz), None, None)
        self.nnz = nnz.value
        self.n_rows, self.n_cols = n_rows, n_cols
        mrl = ctypes.c_int32(0)
        call("skg_pattern_row_groups", h, ctypes.byref(mrl))
        # the fixed-order row-group passes (and their chunked host outputs) serve
        # this pattern; otherwise assemblies gather per row from global memory
        self.row_groups = mrl.value > 0

    def device_csr(self):
        """(crow_indices, col_indices) int64 CUDA tensors of the pattern (cached)."""
        if getattr(self, "_dev_csr", None) is None:
            indptr = dev.empty(self.n_rows + 1, np.int64)
            indices = dev.empty(max(1, self.nnz), np.int32)
            call("skg_pattern_export", self.h, dev.ptr(indptr), dev.ptr(indices), dev.stream_ptr())
            self._dev_csr = (indptr, indices[: self.nnz].long())
        return self._dev_csr

    def host_csr(self):
        indptr = dev.empty(self.n_rows + 1, np.int64)
        indices = dev.empty(max(1, self.nnz), np.int32)
        call("skg_pattern_export", self.h, dev.ptr(indptr), dev.ptr(indices), dev.stream_ptr())
        return indptr.cpu().numpy(), indices[: self.nnz].cpu().numpy()

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            try:
                from ._native import load

                load().skg_pattern_destroy(h)
            except Exception:
                pass
            self.h = None


def per_element(c, E, Q, name):
    """(E,) values when ``c`` (broadcastable to (E, Q)) is constant over the
    points of every element, else None; a scalar stays a 0-d array (callers
    pass no array at all for the scalar 1, the kernels' default)."""
    c = np.asarray(c, dtype=np.float64)
    if c.ndim == 0:
        return c
    try:
        b = np.broadcast_to(c, (E, Q))
    except ValueError as error:
        raise ValueError(f"{name} coefficient must broadcast to {(E, Q)}") from error
    if Q == 1 or b.strides[1] == 0 or np.array_equal(b, b[:, :1] * np.ones((1, Q))):
        return np.ascontiguousarray(b[:, 0])
    return None


def per_point(c, E, Q, name):
    c = np.asarray(c, dtype=np.float64)
    try:
        return np.ascontiguousarray(np.broadcast_to(c, (E, Q)))
    except ValueError as error:
        raise ValueError(f"{name} coefficient must broadcast to {(E, Q)}") from error


def anisotropic_tensor(raw, E, Q, dim=3):
    """(3,3) | (3,3,E,Q) public | (E,Q,3,3) native -> (E,Q,3,3) view
    (forms.py:377-404)."""
    tensor = np.asarray(raw, dtype=np.float64)
    shape = (E, Q)
    if tensor.shape == (dim, dim):
        return np.broadcast_to(tensor, shape + (dim, dim))
    if tensor.shape == (dim, dim) + shape:
        return np.moveaxis(tensor, (0, 1), (-2, -1))
    if tensor.shape == shape + (dim, dim):
        return tensor
    raise ValueError(
        "anisotropic tensor must use the recommended scikit-fem shape "
        f"{(dim, dim) + shape}, constant shape ({dim}, {dim}), or the low-level native "
        f"compatibility shape {shape + (dim, dim)}; got {tensor.shape}")


def tensor_per_element(raw, E, Q, dim=3):
    """Per-element view of a tensor coefficient constant over the points of
    each element, as (array, coef_kind): coef_kind 2 for the public
    component-first layout (3, 3, E), 1 for (E, 3, 3).  None when the tensor
    varies over points."""
    A = np.asarray(raw, dtype=np.float64)
    if A.shape == (dim, dim):
        return np.broadcast_to(A, (E, dim, dim)), 1
    if A.shape == (dim, dim, E, Q):
        if Q == 1 or A.strides[3] == 0 or np.array_equal(A, np.broadcast_to(A[..., :1], A.shape)):
            return A[..., 0], 2
        return None
    if A.shape == (E, Q, dim, dim):
        if Q == 1 or A.strides[1] == 0 or np.array_equal(A, np.broadcast_to(A[:, :1], A.shape)):
            return A[:, 0], 1
        return None
    anisotropic_tensor(A, E, Q, dim)  # raises the shape error
    return None


class _Staging:
    """Pinned host buffer + device buffer for per-call coefficient uploads
    (host copy into page-locked memory, then one asynchronous H2D copy)."""

    def __init__(self):
        self.n = 0
        self.h = self.hv = self.d = None
        self.done = None  # event recorded after the last H2D copy

    def upload(self, a):
        import torch

        a = np.asarray(a, dtype=np.float64)
        n = a.size
        if self.done is not None:
            self.done.synchronize()  # the previous copy has left the pinned buffer
        if n > self.n:
            self.h, self.hv = dev.pinned_empty(n)
            self.d = dev.empty(n, np.float64)
            self.n = n
        self.h[:n].view(a.shape).copy_(dev.host_tensor(a))  # parallel CPU copy
        self.d[:n].copy_(self.h[:n], non_blocking=True)
        self.done = torch.cuda.Event()
        self.done.record()
        return self.d


class _MatrixTarget:
    """Device values + reused host CSR matrix sharing one pinned buffer."""

    def __init__(self, pattern, shape):
        self.pattern = pattern
        indptr, indices = pattern.host_csr()
        self.d_values = dev.empty(max(1, pattern.nnz), np.float64)
        self._pinned, host = dev.pinned_empty(max(1, pattern.nnz))
        self.matrix = csr_matrix((host[: pattern.nnz], indices, indptr), shape=shape, copy=False)

    def enqueue_download(self):
        """Queue the copy of the device values into the host matrix's page-locked values."""
        self._pinned[: self.pattern.nnz].copy_(self.d_values[: self.pattern.nnz], non_blocking=True)

    def download(self):
        import torch

        self.enqueue_download()
        torch.cuda.current_stream().synchronize()
        return self.matrix

    def torch_csr(self):
        """The device values as a CUDA ``torch.sparse_csr_tensor`` (no host copy;
        the values buffer is reused by the next assembly, like the host matrix)."""
        import warnings

        import torch

        crow, col = self.pattern.device_csr()
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", UserWarning)  # torch marks sparse CSR as beta
            return torch.sparse_csr_tensor(crow, col, self.d_values[: self.pattern.nnz], size=self.matrix.shape)

    def pinned_ptr(self):
        """Pointer to the page-locked buffer behind the host matrix (copy target)."""
        return ctypes.c_void_p(self._pinned.data_ptr())

    def finish_direct(self):
        import torch

        torch.cuda.current_stream().synchronize()
        return self.matrix

    def copy_matrix(self):
        """Independent copy of the host matrix (multithreaded copies)."""
        m = self.matrix
        return csr_matrix((dev.host_copy(m.data), dev.host_copy(m.indices), dev.host_copy(m.indptr)), shape=m.shape,
                          copy=False)


class AssemblyGraph:
    """An assembly captured into a CUDA graph, for repeated assemblies whose
    inputs change in place (a time loop updating a coefficient between steps):
    ``replay()`` recomputes the matrix values from the current contents of the
    device tensors the capture read, as one graph launch instead of the
    per-call host work (argument checks, tables, a dozen launches).  Capture
    covers the FP64 fused affine path; one plain call runs first (it builds the
    device tables and sets kernel attributes, which a capture may not do)."""

    def __init__(self, launch, target):
        import torch

        launch()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            launch()
        self.target = target

    def replay(self):
        """Re-run the captured assembly on the current stream; returns the device values."""
        self.graph.replay()
        return self.target.d_values


def _device_tensor(t, shape, name):
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError(f"{name} must be a contiguous float64 CUDA tensor")
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)}")
    return t


class NativeBilinearForm:
    """value / gradient / symmetric-gradient / divergence assembly on one basis."""

    def __init__(self, basis, *, memory_limit_bytes=None, memory_safety_factor=1.25):
        self.memory_estimate = estimate_bilinear_memory(basis)
        enforce_memory_budget(self.memory_estimate, memory_limit_bytes, safety_factor=memory_safety_factor)
        self.basis = basis
        E, L = basis.mesh.nelements, basis._nodes * basis._comp
        dofs = basis._dev_dofs()
        self.pattern = Pattern(dofs, dofs, E, L, L, basis.N, basis.N)
        self.target = _MatrixTarget(self.pattern, (basis.N, basis.N))

    @property
    def matrix(self):
        return self.target.matrix

    def _affine_coefficient(self, value, gradient, symmetric_gradient, divergence):
        """(E,) gradient coefficient when the fused affine path applies, else None."""
        b = self.basis
        E, Q = b._coefficient_shape
        if value is None and gradient is None and symmetric_gradient is None and divergence is None:
            raise ValueError("at least one coefficient is required")
        if (b._comp == 1 and value is None and symmetric_gradient is None and divergence is None
                and b.is_affine):
            return per_element(gradient, E, Q, "gradient")
        return None

    def _affine(self, fast, prec, out, host):
        """Fused affine assembly into `out` (device or, with `host`, page-locked host
        memory); the coefficient is read in place from host memory when possible
        (the caller then synchronises before `fast` goes away)."""
        b = self.basis
        E, Q = b._coefficient_shape
        coef = keep = None
        if np.ndim(fast) == 0:
            fast = None if float(fast) == 1.0 else np.full(E, float(fast))
        if fast is not None:
            coef = dev.host_readable(fast) if host else None
            if coef is None:
                keep = dev.to_device(fast, np.float64)
                coef = dev.ptr(keep)
        if host:  # values to the host matrix: copies overlap the row pass
            call("skg_h1_assemble_affine_host", self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1],
                 dev.ptr(b.mesh._dev("t")), b._nodes, E, Q, dev.hptr(b.X),
                 dev.hptr(b.W), 0, coef, prec, dev.ptr(self.target.d_values), out, dev.stream_ptr())
        else:
            call("skg_h1_assemble_affine", self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1],
                 dev.ptr(b.mesh._dev("t")), b._nodes, E, Q, dev.hptr(b.X),
                 dev.hptr(b.W), 0, coef, prec, out, dev.stream_ptr())
        return keep

    def capture_gradient(self, kappa):
        """CUDA-graph capture of ``gradient=kappa`` (per-element FP64 CUDA tensor,
        shape (E,)) on an affine scalar basis: returns an ``AssemblyGraph`` whose
        ``replay()`` reassembles the device values for the current ``kappa``."""
        b = self.basis
        if b._comp != 1 or not b.is_affine:
            raise UnsupportedNativeForm("graph capture covers the affine scalar gradient path")
        E, Q = b._coefficient_shape
        kappa = _device_tensor(kappa, (E,), "kappa")

        def launch():
            call("skg_h1_assemble_affine", self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1],
                 dev.ptr(b.mesh._dev("t")), b._nodes, E, Q, dev.hptr(b.X),
                 dev.hptr(b.W), 0, dev.ptr(kappa), SKG_FP64, dev.ptr(self.target.d_values), dev.stream_ptr())

        return AssemblyGraph(launch, self.target)

    def assemble_device(self, *, value=None, gradient=None, symmetric_gradient=None, divergence=None,
                        precision="fp64"):
        """Assemble into the device values (no host copy); returns the device tensor."""
        b = self.basis
        E, Q = b._coefficient_shape
        prec = _precision(precision)
        fast = self._affine_coefficient(value, gradient, symmetric_gradient, divergence)
        if fast is not None:
            self._affine(fast, prec, dev.ptr(self.target.d_values), host=False)
            return self.target.d_values
        if prec != SKG_FP64:
            raise UnsupportedNativeForm("split precision is available on the affine scalar gradient path")
        forms = self._p1_forms(value, gradient, symmetric_gradient, divergence)
        if forms is not None:
            self._p1_forms_launch(forms, dev.ptr(self.target.d_values), None)
            return self.target.d_values
        tab = b._device_tabulation()
        coefs = [self._point_coefficient(c, E, Q, n)
                 for c, n in ((value, "value"), (gradient, "gradient"),
                              (symmetric_gradient, "symmetric_gradient"), (divergence, "divergence"))]
        call("skg_h1_assemble_tabulated", self.pattern.h, dev.ptr(b._dev_dofs()), E, b._nodes, b._comp, Q,
             dev.ptr(tab["shape"]), dev.ptr(tab["grad"]), dev.ptr(tab["dx"]), *(dev.ptr(c) for c in coefs),
             dev.ptr(self.target.d_values), None, dev.stream_ptr())
        return self.target.d_values

    def _p1_forms(self, value, gradient, symmetric_gradient, divergence):
        """The four coefficients as (E,) arrays, 0-d scalars or None when the
        fused P1 path applies (affine P1 basis with 1 or 3 components, every
        coefficient constant on each element, row-grouped pattern), else None."""
        b = self.basis
        if b._nodes != 4 or b._comp not in (1, 3) or not b.is_affine or not self.pattern.row_groups:
            return None
        E, Q = b._coefficient_shape
        out = []
        for c, name in ((value, "value"), (gradient, "gradient"),
                        (symmetric_gradient, "symmetric_gradient"), (divergence, "divergence")):
            if c is None:
                out.append(None)
                continue
            if hasattr(c, "is_cuda"):
                return None  # torch tensors of point values: the tabulated path reads them in place
            pe = per_element(c, E, Q, name)
            if pe is None:
                return None
            out.append(pe)
        return out

    def _p1_forms_launch(self, forms, d_values, h_values):
        """skg_p1_assemble_affine_forms; per-element arrays are read in place
        from host memory when `h_values` is given (the caller synchronises
        before the arrays go away), else uploaded.  Returns the uploads."""
        b = self.basis
        E, Q = b._coefficient_shape
        ptrs, consts, keep = [], [], []
        for c in forms:
            if c is None or np.ndim(c) == 0:
                ptrs.append(None)
                consts.append(0.0 if c is None else float(c))
                continue
            ptr = dev.host_readable(c) if h_values is not None else None
            if ptr is None:
                keep.append(dev.to_device(c, np.float64))
                ptr = dev.ptr(keep[-1])
            ptrs.append(ptr)
            consts.append(0.0)
        call("skg_p1_assemble_affine_forms", self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1],
             dev.ptr(b.mesh._dev("t")), E, b._comp, Q, dev.hptr(b.X), dev.hptr(b.W), *ptrs, *consts,
             d_values, h_values, dev.stream_ptr())
        return keep

    def _point_coefficient(self, c, E, Q, name):
        """(E, Q) float64 device array for a coefficient: a CUDA tensor of that
        shape is used as is, a scalar becomes a cached device constant (no
        host-to-device copy per call), anything else is broadcast and uploaded."""
        if c is None:
            return None
        if hasattr(c, "is_cuda") and c.is_cuda:
            return _device_tensor(c, (E, Q), name)
        a = np.asarray(c, dtype=np.float64)
        if a.ndim == 0:
            import torch

            cache = self.__dict__.setdefault("_constants", {})
            t = cache.get(float(a))
            if t is None:
                if len(cache) >= 8:
                    cache.clear()
                t = cache[float(a)] = torch.full((E, Q), float(a), dtype=torch.float64, device="cuda")
            return t
        return dev.to_device(per_point(a, E, Q, name), np.float64)

    def assemble_torch(self, *, value=None, gradient=None, symmetric_gradient=None, divergence=None,
                       precision="fp64"):
        """Device-resident result for GPU consumers: a CUDA sparse CSR tensor."""
        self.assemble_device(value=value, gradient=gradient, symmetric_gradient=symmetric_gradient,
                             divergence=divergence, precision=precision)
        return self.target.torch_csr()

    def assemble(self, *, value=None, gradient=None, symmetric_gradient=None, divergence=None,
                 num_threads=0, precision="fp64"):
        """Host CSR matrix (reused between calls, as the reference's).  On the fused
        path the kernels write the values straight into its page-locked buffer."""
        fast = self._affine_coefficient(value, gradient, symmetric_gradient, divergence)
        if fast is not None:
            self._affine(fast, _precision(precision), self.target.pinned_ptr(), host=True)
            return self.target.finish_direct()
        forms = self._p1_forms(value, gradient, symmetric_gradient, divergence)
        if forms is not None and _precision(precision) == SKG_FP64:
            self._p1_forms_launch(forms, dev.ptr(self.target.d_values), self.target.pinned_ptr())
            return self.target.finish_direct()
        self.assemble_device(value=value, gradient=gradient, symmetric_gradient=symmetric_gradient,
                             divergence=divergence, precision=precision)
        return self.target.download()


class NativeTensorForm:
    """dot(mul(A, grad u), grad v) on one scalar basis (NativeCrossBilinearForm
    .assemble_tensor("gradient", "gradient", ...), bilinear_form.py:336-367)."""

    def __init__(self, basis, *, memory_limit_bytes=None, memory_safety_factor=1.25):
        if basis._comp != 1:
            raise UnsupportedNativeForm("anisotropic gradient tensor currently requires a scalar field")
        self.memory_estimate = estimate_bilinear_memory(basis)
        enforce_memory_budget(self.memory_estimate, memory_limit_bytes, safety_factor=memory_safety_factor)
        self.basis = basis
        E, L = basis.mesh.nelements, basis._nodes
        dofs = basis._dev_dofs()
        self.pattern = Pattern(dofs, dofs, E, L, L, basis.N, basis.N)
        self.target = _MatrixTarget(self.pattern, (basis.N, basis.N))
        self._staging = _Staging()

    def assemble_device(self, raw, precision="fp64", tensor_device=None, tensor_kind=2):
        """Assemble into the device values.  ``tensor_device``: a per-element
        float64 device tensor already resident, (3,3,E) for tensor_kind 2 or
        (E,3,3) for tensor_kind 1 (skips the host upload)."""
        self._run(raw, precision, tensor_device, tensor_kind, None)
        return self.target.d_values

    def _run(self, raw, precision, tensor_device, tensor_kind, out):
        """Launch the assembly; with `out` (host values pointer) the fused path
        writes there and reads a per-element tensor in place from host memory.
        Returns True when the values went to `out`."""
        b = self.basis
        E, Q = b._coefficient_shape
        prec = _precision(precision)
        kind = tensor_kind
        coef = keep = None
        if tensor_device is not None:
            coef = dev.ptr(tensor_device)
        elif b.is_affine:
            pe = tensor_per_element(raw, E, Q)
            if pe is not None:
                arr, kind = pe
                coef = dev.host_readable(arr) if out is not None else None
                if coef is None:
                    keep = self._staging.upload(arr)
                    coef = dev.ptr(keep)
        if coef is not None:
            if out is not None:  # values to the host matrix: copies overlap the row pass
                call("skg_h1_assemble_affine_host", self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1],
                     dev.ptr(b.mesh._dev("t")), b._nodes, E, Q, dev.hptr(b.X),
                     dev.hptr(b.W), kind, coef, prec, dev.ptr(self.target.d_values), out, dev.stream_ptr())
                return True
            call("skg_h1_assemble_affine", self.pattern.h, dev.ptr(b.mesh._dev("p")), b.mesh.p.shape[1],
                 dev.ptr(b.mesh._dev("t")), b._nodes, E, Q, dev.hptr(b.X),
                 dev.hptr(b.W), kind, coef, prec, dev.ptr(self.target.d_values), dev.stream_ptr())
            return False
        if prec != SKG_FP64:
            raise UnsupportedNativeForm("split precision is available on the affine tensor path")
        T = anisotropic_tensor(raw, E, Q)
        tab = b._device_tabulation()
        d = self._staging.upload(T)
        call("skg_h1_assemble_tensor_tabulated", self.pattern.h, dev.ptr(b._dev_dofs()), E, b._nodes, 1, Q,
             dev.ptr(tab["grad"]), dev.ptr(tab["dx"]), dev.ptr(d), dev.ptr(self.target.d_values), None,
             dev.stream_ptr())
        return False

    def assemble_torch(self, raw, precision="fp64"):
        """Device-resident result for GPU consumers: a CUDA sparse CSR tensor."""
        self.assemble_device(raw, precision)
        return self.target.torch_csr()

    def capture(self, tensor_device, tensor_kind=2):
        """CUDA-graph capture of the FP64 assembly with a per-element tensor
        already on the device ((3, 3, E) for tensor_kind 2, (E, 3, 3) for 1):
        returns an ``AssemblyGraph`` whose ``replay()`` reassembles the device
        values for the tensor's current contents."""
        b = self.basis
        if not b.is_affine:
            raise UnsupportedNativeForm("graph capture covers affine bases")
        E = b.mesh.nelements
        _device_tensor(tensor_device, (3, 3, E) if tensor_kind == 2 else (E, 3, 3), "tensor_device")
        return AssemblyGraph(lambda: self._run(None, "fp64", tensor_device, tensor_kind, None), self.target)

    def assemble(self, raw, precision="fp64", copy=True):
        """Host CSR matrix.  ``copy=True`` (the reference's behaviour,
        bilinear_form.py:367) returns an independent matrix; ``copy=False`` the
        reused one whose page-locked values the fused kernels write directly."""
        direct = self._run(raw, precision, None, 2, self.target.pinned_ptr())
        m = self.target.finish_direct() if direct else self.target.download()
        return self.target.copy_matrix() if copy else m


class NativeCrossBilinearForm:
    """Test x trial assembly between two bases of one mesh and one quadrature
    rule (NativeCrossBilinearForm, bilinear_form.py:102-367): value, gradient
    and divergence kinds, and caller-supplied value / gradient contraction
    tensors.  Each call returns a new matrix, as the reference's."""

    def __init__(self, test_basis, trial_basis, *, memory_limit_bytes=None, memory_safety_factor=1.25):
        # the budget first: reading dx below makes the bases' device tabulation
        self.memory_estimate = estimate_bilinear_memory(test_basis, trial_basis)
        enforce_memory_budget(self.memory_estimate, memory_limit_bytes, safety_factor=memory_safety_factor)
        if test_basis.dx.shape != trial_basis.dx.shape:
            raise ValueError("trial and test quadrature shapes must match")
        if not np.allclose(test_basis.dx, trial_basis.dx):
            raise ValueError("trial and test quadrature weights must match")
        if not np.allclose(test_basis.global_coordinates, trial_basis.global_coordinates):
            raise ValueError("trial and test quadrature coordinates must match")
        self.test_basis, self.trial_basis = test_basis, trial_basis
        E = test_basis.mesh.nelements
        Lt, Lc = test_basis._nodes * test_basis._comp, trial_basis._nodes * trial_basis._comp
        self.pattern = Pattern(test_basis._dev_dofs(), trial_basis._dev_dofs(), E, Lt, Lc, test_basis.N,
                               trial_basis.N)
        self.target = _MatrixTarget(self.pattern, (test_basis.N, trial_basis.N))
        self.shape = (test_basis.N, trial_basis.N)
        self.coefficient_shape = test_basis.dx.shape
        self.test_components = test_basis._comp
        self.trial_components = trial_basis._comp
        self.dimension = 3
        # facet normals of the bases (bilinear_form.py:177-178): None for volume bases
        self.test_normals = getattr(test_basis, "normals", None)
        self.trial_normals = getattr(trial_basis, "normals", None)

    def assemble(self, kind, coefficient):
        """kind: "value", "gradient", "row_divergence" (vector test, scalar
        trial) or "column_divergence" (scalar test, vector trial); coefficient
        broadcast to the (cell, point) shape."""
        coefficient = np.asarray(coefficient, dtype=np.float64)
        scalar = np.broadcast_to(coefficient, self.coefficient_shape)
        Ct, Cc, d = self.test_components, self.trial_components, self.dimension
        if kind in ("row_divergence", "column_divergence"):
            if kind == "row_divergence":
                if Ct != d or Cc != 1:
                    raise ValueError("row divergence requires vector test and scalar trial")
                tensor = np.zeros((Ct, d, Cc))
                for comp in range(Ct):
                    tensor[comp, comp, 0] = 1.0
                row_kind, column_kind = "gradient", "value"
            else:
                if Cc != d or Ct != 1:
                    raise ValueError("column divergence requires scalar test and vector trial")
                tensor = np.zeros((Ct, Cc, d))
                for comp in range(Cc):
                    tensor[0, comp, comp] = 1.0
                row_kind, column_kind = "value", "gradient"
        else:
            if Ct != Cc:
                raise ValueError("value and gradient contractions require matching component counts")
            if kind == "gradient":
                tensor = np.einsum("rc,ij->ricj", np.eye(Ct), np.eye(d))
                row_kind = column_kind = "gradient"
            else:
                tensor = np.eye(Ct)
                row_kind = column_kind = "value"
        full = scalar[(...,) + (None,) * tensor.ndim] * tensor
        return self.assemble_tensor(row_kind, column_kind, full)

    def assemble_kinds(self, row_kind, column_kind, coefficient=1.0, *, num_threads=0):
        """Value / gradient contractions with a scalar coefficient c
        (bilinear_form.py:244-334) on volume bases, component by component:
        value-value c; a gradient against a value pairs each derivative
        direction with the value, c for every direction; gradient-gradient c
        for equal directions.  ``normal_gradient`` needs facet normals, which
        volume bases do not have (ValueError, as the reference's)."""
        valid = {"value", "gradient", "normal_gradient"}
        if row_kind not in valid or column_kind not in valid:
            raise ValueError("cross kind must be value, gradient, or normal_gradient")
        if self.test_components != self.trial_components:
            raise ValueError("cross contractions require matching components")
        scalar = np.broadcast_to(np.asarray(coefficient, dtype=np.float64), self.coefficient_shape)
        if row_kind == "normal_gradient" and self.test_normals is None:
            raise ValueError("row normal_gradient requires test-basis normals")
        if column_kind == "normal_gradient" and self.trial_normals is None:
            raise ValueError("column normal_gradient requires trial-basis normals")
        if "normal_gradient" in (row_kind, column_kind):
            raise UnsupportedNativeForm("normal_gradient contractions need facet bases")
        C, d = self.test_components, self.dimension
        if row_kind == "value" and column_kind == "value":
            pattern = np.eye(C)
        elif column_kind == "value":
            pattern = np.einsum("rc,i->ric", np.eye(C), np.ones(d))
        elif row_kind == "value":
            pattern = np.einsum("rc,j->rcj", np.eye(C), np.ones(d))
        else:
            pattern = np.einsum("rc,ij->ricj", np.eye(C), np.eye(d))
        # the coefficient placed into zeros (exact zeros elsewhere, whatever its sign)
        tensor = np.zeros(self.coefficient_shape + pattern.shape)
        for index in zip(*np.nonzero(pattern)):
            tensor[(Ellipsis,) + index] = scalar
        return self.assemble_tensor(row_kind, column_kind, tensor, num_threads=num_threads)

    def assemble_tensor(self, row_kind, column_kind, coefficient, *, num_threads=0):
        """Assemble a caller-supplied value / gradient contraction tensor
        (cell, point) + row axes + column axes."""
        valid = {"value", "gradient"}
        if row_kind not in valid or column_kind not in valid:
            raise ValueError("tensor kind must be value or gradient")
        row_axes = (self.test_components,) + ((self.dimension,) if row_kind == "gradient" else ())
        column_axes = (self.trial_components,) + ((self.dimension,) if column_kind == "gradient" else ())
        expected = self.coefficient_shape + row_axes + column_axes
        coefficient = np.asarray(coefficient, dtype=np.float64)
        try:
            coefficient = np.broadcast_to(coefficient, expected)
        except ValueError as error:
            raise ValueError(f"tensor coefficient must broadcast to {expected}") from error
        tb, cb = self.test_basis, self.trial_basis
        tt, ct = tb._device_tabulation(), cb._device_tabulation()
        E, Q = self.coefficient_shape
        d_coef = dev.to_device(coefficient, np.float64)
        call("skg_cross_assemble_tabulated", self.pattern.h, E, Q, tb._nodes, tb._comp,
             int(row_kind == "gradient"), dev.ptr(tt["shape"]), dev.ptr(tt["grad"]), cb._nodes, cb._comp,
             int(column_kind == "gradient"), dev.ptr(ct["shape"]), dev.ptr(ct["grad"]), dev.ptr(tt["dx"]),
             dev.ptr(d_coef), dev.ptr(self.target.d_values), dev.stream_ptr())
        self.target.download()
        return self.target.copy_matrix()


@dataclass(frozen=True)
class LinearFormDiagnostics:
    """What ``NativeLinearForm.assemble`` reports beside the vector
    (linear_form.py:10-14): elements, points per element, and the wall time of
    the call (coefficient upload, kernels, copy of the result)."""

    entity_count: int
    quadrature_point_count: int
    assembly_seconds: float


class NativeLinearForm:
    """f.v + G:grad v on one basis (linear_form.py:17-107).  ``assemble``
    returns (vector, LinearFormDiagnostics) as the reference's does."""

    def __init__(self, basis):
        self.basis = basis
        E, L = basis.mesh.nelements, basis._nodes * basis._comp
        Q = len(basis.W)
        self._shape = (E, Q, basis._comp)
        self._gradient_shape = (E, Q, basis._comp, 3)
        self.pattern = Pattern(basis._dev_dofs(), None, E, L, 0, basis.N, 0)
        self.d_out = dev.empty(max(1, basis.N), np.float64)

    @property
    def ndofs(self):
        return self.basis.N

    @staticmethod
    def _coefficient(name, coefficient, shape):
        """None, a constant of shape ``shape[2:]``, or an array broadcast to
        ``shape``; float64 only (linear_form.py:91-107)."""
        if coefficient is None:
            return None
        coefficient = np.asarray(coefficient)
        if coefficient.dtype != np.float64:
            raise TypeError(f"{name} coefficient must have dtype float64")
        if coefficient.shape == shape[2:]:
            return np.ascontiguousarray(coefficient)
        try:
            return np.broadcast_to(coefficient, shape)
        except ValueError as error:
            raise ValueError(f"{name} coefficient must broadcast to {shape}") from error

    def assemble(self, *, value=None, gradient=None, num_threads=0):
        start = time.perf_counter()
        b = self.basis
        E, Q, C = self._shape
        value = self._coefficient("value", value, self._shape)
        gradient = self._coefficient("gradient", gradient, self._gradient_shape)
        if value is None and gradient is None:
            raise ValueError("at least one coefficient is required")
        dv = dg = None
        if value is not None:
            dv = dev.to_device(np.ascontiguousarray(np.broadcast_to(value, self._shape)), np.float64)
        if gradient is not None:
            dg = dev.to_device(np.ascontiguousarray(np.broadcast_to(gradient, self._gradient_shape)), np.float64)
        tab = b._device_tabulation()
        call("skg_linear_assemble_tabulated", self.pattern.h, dev.ptr(b._dev_dofs()), E, b._nodes, C, Q,
             dev.ptr(tab["shape"]), dev.ptr(tab["grad"]), dev.ptr(tab["dx"]), dev.ptr(dv), dev.ptr(dg),
             dev.ptr(self.d_out), dev.stream_ptr())
        result = self.d_out[: b.N].cpu().numpy()
        return result, LinearFormDiagnostics(E, Q, time.perf_counter() - start)


def assemble_bilinear(form, basis, terms, *, precision="fp64", memory_limit_bytes=None,
                      memory_safety_factor=1.25):
    plain = {"value": None, "gradient": None, "symmetric_gradient": None, "divergence": None}
    tensors = []
    for kind, coef in terms:
        if kind in plain:
            plain[kind] = coef if plain[kind] is None else plain[kind] + coef
        elif kind == "gradient_tensor":
            tensors.append(coef)
        else:
            raise UnsupportedNativeForm(f"unsupported bilinear term kind {kind!r}")
    result = None
    if any(v is not None for v in plain.values()):
        native = form._native_cache.get(basis)
        if native is None:
            native = NativeBilinearForm(basis, memory_limit_bytes=memory_limit_bytes,
                                        memory_safety_factor=memory_safety_factor)
            form._native_cache[basis] = native
        elif memory_limit_bytes is not None:
            enforce_memory_budget(native.memory_estimate, memory_limit_bytes, safety_factor=memory_safety_factor)
        result = native.assemble(precision=precision, **plain)
    if tensors:
        tnative = form._tensor_cache.get(basis)
        if tnative is None:
            tnative = NativeTensorForm(basis, memory_limit_bytes=memory_limit_bytes,
                                       memory_safety_factor=memory_safety_factor)
            form._tensor_cache[basis] = tnative
        for raw in tensors:
            m = tnative.assemble(raw, precision)
            result = m if result is None else result + m
    if result is None:
        raise UnsupportedNativeForm("bilinear form contains no assembled terms")
    return result


def assemble_linear(form, basis, terms):
    native = form._native_cache.get(basis)
    if native is None:
        native = NativeLinearForm(basis)
        form._native_cache[basis] = native
    E, Q = basis._coefficient_shape
    C = basis._comp
    value = gradient = None
    for kind, c in terms:
        c = np.asarray(c, dtype=np.float64)
        if kind == "value":
            if C == 1 and c.shape == (E, Q):
                c = c[..., None]
            elif c.ndim and c.shape[0] == C and c.shape != (C,):
                c = np.moveaxis(c, 0, -1)
            value = c if value is None else value + c
        elif kind == "gradient":
            if c.ndim >= 2 and c.shape[:2] == (C, 3):
                c = np.moveaxis(c, (0, 1), (-2, -1))
            gradient = c if gradient is None else gradient + c
        else:
            raise UnsupportedNativeForm
    result, _ = native.assemble(value=value, gradient=gradient)
    return result
