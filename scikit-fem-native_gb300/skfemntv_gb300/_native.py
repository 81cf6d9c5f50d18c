"""ctypes binding of the C ABI declared in ``include/skfem_gb300.h``.

The library is the only compute path: when it is missing, or no CUDA device
is present, the first call raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libskfem_gb300.so")

SKG_OK = 0
SKG_EINVAL = 1
SKG_ENOMEM = 2
SKG_ECUDA = 3
SKG_EGEOM = 4
SKG_ERANGE = 5
SKG_EUNSUPPORTED = 6

SKG_FP64 = 0
SKG_SPLIT_FP32 = 1
SKG_FP64_EMULATED = 2

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_i64p = ctypes.POINTER(ctypes.c_int64)

# name -> argument types (all return int status unless listed in _RESTYPE)
SIGNATURES = {
    "skg_version": [],
    "skg_last_error": [],
    "skg_pattern_create": [_vp, _vp, _i64, _i32, _i32, _i64, _i64, _vp, ctypes.POINTER(_vp)],
    "skg_pattern_destroy": [_vp],
    "skg_pattern_info": [_vp, _i64p, _i64p, _i64p],
    "skg_pattern_export": [_vp, _vp, _vp, _vp],
    "skg_geometry_diagnostics": [_vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp],
    "skg_tabulate_geometry": [_vp, _i64, _vp, _i32, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _vp,
                              _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64p, _vp],
    "skg_h1_assemble_tabulated": [_vp, _vp, _i64, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp,
                                  _vp, _vp, _vp, _vp],
    "skg_h1_assemble_tensor_tabulated": [_vp, _vp, _i64, _i32, _i32, _i32, _vp, _vp, _vp, _vp,
                                         _vp, _vp],
    "skg_h1_assemble_affine": [_vp, _vp, _i64, _vp, _i32, _i64, _i32, _vp, _vp, _i32, _vp,
                               _i32, _vp, _vp],
    "skg_h1_assemble_affine_profiled": [_vp, _vp, _i64, _vp, _i32, _i64, _i32, _vp, _vp, _i32,
                                        _vp, _i32, _vp, ctypes.POINTER(ctypes.c_float), _vp],
    "skg_h1_assemble_affine_noalloc": [_vp, _vp, _i64, _vp, _i32, _i64, _i32, _vp, _vp, _i32, _vp, _i32,
                                       _vp, _vp],
    "skg_edge_topology": [_vp, _i64, _vp, _vp, _vp, _i64p, _i64p, _vp],
    "skg_n1_assemble": [_vp, _vp, _i64, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _i32, _i32,
                        _i32, _vp, _vp],
    "skg_n1_assemble_host": [_vp, _vp, _i64, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _i32, _i32,
                             _i32, _vp, _vp, _vp],
    "skg_n1_assemble_pointwise": [_vp, _vp, _i64, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _i32,
                                  _i32, _vp, _vp],
    "skg_p1_energy": [_vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp, ctypes.c_double, _vp, _vp],
    "skg_p1_energy_grad": [_vp, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp, ctypes.c_double,
                           ctypes.c_double, _vp, _vp, _vp, _vp, _vp],
    "skg_p1_energy_value_and_grad": [_vp, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp, ctypes.c_double,
                                     ctypes.c_double, _vp, _vp, _vp, _vp, _vp, _vp],
    "skg_nh_assemble": [_vp, _vp, _i64, _vp, _i64, _vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                        _vp, _vp, _vp],
    "skg_nh_assemble_host": [_vp, _vp, _i64, _vp, _i64, _vp, ctypes.c_double, ctypes.c_double,
                             ctypes.c_double, _vp, _vp, _vp, _vp, _vp],
    "skg_mlp_param_count": [],
    "skg_mlp_dataset": [_i64, ctypes.c_uint64, ctypes.c_double, ctypes.c_double, ctypes.c_double, _vp, _vp, _vp],
    "skg_mlp_loss_grad": [_vp, _vp, _vp, _i64, _vp, _i64, _i32, ctypes.c_float, _vp, _vp, _vp],
    "skg_mlp_train": [_vp, _vp, _vp, _i64, _vp, _i32, _i32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                      _vp, _vp, _i32, ctypes.POINTER(ctypes.c_float), _vp],
    "skg_mlp_refine": [_vp, _vp, _vp, _i64, _vp, _i64, _i32, _i32, _i32, ctypes.c_float,
                       ctypes.POINTER(ctypes.c_double), _vp],
    "skg_mlp_eval": [_vp, _vp, _i64, _vp, _vp],
    "skg_fp64_fma_rate": [_vp, _vp],
    "skg_device_pageable_access": [ctypes.POINTER(ctypes.c_int32)],
    "skg_h1_assemble_affine_host": [_vp, _vp, _i64, _vp, _i32, _i64, _i32, _vp, _vp, _i32, _vp, _i32, _vp, _vp,
                                    _vp],
    "skg_cross_assemble_tabulated": [_vp, _i64, _i32, _i32, _i32, _i32, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp,
                                     _vp, _vp, _vp],
    "skg_n1_vector_load": [_vp, _vp, _i64, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp],
    "skg_n1_element_matrices": [_vp, _i64, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp,
                                _vp],
    "skg_n1_evaluate": [_vp, _i64, _vp, _vp, _vp, _i64, _i64, _i32, _vp, _vp, _i32, _vp, _vp],
    "skg_n1_edge_points": [_vp, _i64, _vp, _i64, _i32, _vp, _vp, _vp],
    "skg_n1_edge_moments": [_vp, _i64, _vp, _i64, _i32, _vp, _vp, _vp, _vp],
    "skg_pattern_row_groups": [_vp, ctypes.POINTER(ctypes.c_int32)],
    "skg_nh_assemble_surrogate": [_vp, _vp, _i64, _vp, _i64, _vp, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_double, _vp, _vp, ctypes.c_float, _vp, _vp, _i64p, _vp],
    "skg_nh_assemble_surrogate_host": [_vp, _vp, _i64, _vp, _i64, _vp, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, _vp, _vp, ctypes.c_float, _vp, _vp, _vp, _vp, _i64p,
                                       _vp],
    "skg_p1_assemble_affine_forms": [_vp, _vp, _i64, _vp, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _vp, _vp,
                                     _vp],
    "skg_linear_assemble_tabulated": [_vp, _vp, _i64, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp,
                                      _vp, _vp],
}
_RESTYPE = {"skg_last_error": ctypes.c_char_p}
_NO_STATUS = {"skg_mlp_param_count", "skg_version"}

_lib = None


class NativeError(RuntimeError):
    pass


def load():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"skfemntv_gb300 native library not built ({LIB_PATH}); run "
            "scikit-fem-native_gb300/build_native.py"
        )
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPE.get(name, ctypes.c_int)
    _lib = lib
    return lib


def exported_symbols():
    return list(SIGNATURES)


def last_error() -> str:
    msg = load().skg_last_error()
    return msg.decode() if msg else ""


def check(status: int):
    """Map a C ABI status to the exception type the reference raises."""
    if status == SKG_OK:
        return
    msg = last_error()
    if status in (SKG_EINVAL, SKG_EGEOM, SKG_ERANGE):
        raise ValueError(msg)
    if status == SKG_ENOMEM:
        raise MemoryError(msg)
    if status == SKG_EUNSUPPORTED:
        from .errors import UnsupportedNativeForm

        raise UnsupportedNativeForm(msg)
    raise NativeError(msg)


def call(name: str, *args):
    result = getattr(load(), name)(*args)
    if name not in _NO_STATUS:
        check(result)
    return result
