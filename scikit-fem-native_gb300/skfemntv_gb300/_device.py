"""Device memory and stream plumbing (PyTorch provides allocation and streams).

Nothing here computes: arrays are moved between host and device and their
raw pointers handed to the C ABI.  All device work requires CUDA; without a
GPU the helpers raise.
"""
from __future__ import annotations

import ctypes

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover - torch is part of the runtime image
    torch = None


def require_cuda():
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError("skfemntv_gb300 needs a CUDA device (GB300); none is available")
    return torch


def device():
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    """Raw cudaStream_t of PyTorch's current stream."""
    require_cuda()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def hptr(a):
    """Raw pointer of a host array the C ABI reads in C order."""
    if a is None:
        return None
    if not a.flags.c_contiguous:
        raise ValueError("host array passed to the native library must be C-contiguous")
    return a.ctypes.data_as(ctypes.c_void_p)


_TORCH_DTYPES = {
    np.dtype(np.float64): "float64",
    np.dtype(np.float32): "float32",
    np.dtype(np.int32): "int32",
    np.dtype(np.int64): "int64",
    np.dtype(np.int8): "int8",
}


def to_device(a, dtype):
    """Copy a host array to a new contiguous device tensor of ``dtype``."""
    t = require_cuda()
    a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
    if not a.flags.writeable:
        a = a.copy()
    return t.from_numpy(a).to(device(), non_blocking=False)


def empty(shape, dtype):
    t = require_cuda()
    return t.empty(shape, dtype=getattr(t, _TORCH_DTYPES[np.dtype(dtype)]), device=device())


def pinned_empty(n, dtype=np.float64):
    """Page-locked host buffer and its numpy view (fast D2H targets)."""
    t = require_cuda()
    buf = t.empty(n, dtype=getattr(t, _TORCH_DTYPES[np.dtype(dtype)]), pin_memory=True)
    return buf, buf.numpy()


_PAGEABLE = {}


def pageable_access():
    """True when kernels on the current device can read / write pageable host
    memory directly (Grace-Blackwell address translation over NVLink-C2C)."""
    require_cuda()
    d = torch.cuda.current_device()
    if d not in _PAGEABLE:
        from ._native import call

        v = ctypes.c_int32(0)
        call("skg_device_pageable_access", ctypes.byref(v))
        _PAGEABLE[d] = bool(v.value)
    return _PAGEABLE[d]


def host_readable(a):
    """Pointer a kernel can read `a` (float64, C order) through, without a
    copy, or None: needs pageable access and a C-contiguous float64 array.
    The caller keeps `a` alive and synchronises before returning."""
    if a is None or not pageable_access():
        return None
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def host_tensor(a):
    """CPU torch view of a C-contiguous host array (no copy; read-only arrays
    are viewed as well, the view is only read)."""
    import warnings

    t = require_cuda()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return t.from_numpy(np.ascontiguousarray(a))


def host_copy(a):
    """Multithreaded copy of a host array (torch's parallel CPU copy)."""
    t = require_cuda()
    out = np.empty(a.shape, dtype=a.dtype)
    if a.size:
        t.from_numpy(out).copy_(host_tensor(a))
    return out
