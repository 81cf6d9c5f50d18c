"""Allocation-free memory estimates and budgets (python/skfemntv/preflight.py
:18-352), restated for the GPU backend.

The estimate keeps the reference's field names; each field counts what this
backend allocates for the same purpose.  With E elements, Q points per
element, Lr x Lc local DOFs, R rows and nnz the adjacency-free bound
min(rows * columns, E * Lr * Lc):

basis_bytes
    arrays the bases already hold: host DOF numbering, node coordinates and
    quadrature rule; on the device the mesh copies, the geometry checks, and
    the DOF map and tabulation once made.
native_tabulation_bytes
    the device tabulation that the per-point kernels make on first use
    (shape values, gradients, dx, points and geometry checks: 4n + 7 float64
    per point for n nodes), and for a cross form the host copies of dx and
    the points it compares; 0 once the basis holds them.
dof_map_bytes
    int32 element DOF maps on the device: a basis's map until it is made and
    the pattern's copies of the row and column maps.
csr_bytes_upper_bound
    the device CSR (int32 offsets and columns, float64 values), the
    page-locked host matrix (float64 values, int32 columns, int64 offsets)
    and one returned copy of it.
scatter_bytes
    the element matrices one assembly writes and then sums by rows, float64
    E x Lr x Lc.  They are released after each call into the device's memory
    pool, which keeps them reserved, so they count as persistent.
coloring_bytes_upper_bound
    the row-incidence structure that takes the place of the reference's
    element colouring: the int32 incidence list and offsets, one 16-byte
    record per incidence and the row groups (at most R, in two orders).
pattern_temporary_bytes_upper_bound
    device counters and host row lists of the pattern build, and the
    temporaries of the CSR export.
staging_bytes_upper_bound
    per call: the per-element geometry of the scalar affine path (16 float64
    per element) and the page-locked and device copies of per-point
    coefficients.  The reference has no such field: its kernels read the
    caller's arrays.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, fields, is_dataclass

import numpy as np

_I32, _I64, _F64 = 4, 8, 8


def format_bytes(count: int) -> str:
    value = float(count)
    for unit in ("B", "KiB", "MiB", "GiB", "TiB"):
        if value < 1024.0 or unit == "TiB":
            return f"{value:.1f} {unit}"
        value /= 1024.0
    raise AssertionError("unreachable")


@dataclass(frozen=True)
class AssemblyMemoryEstimate:
    """Conservative memory estimate made before an assembler is constructed.

    ``basis_bytes`` are already held by the bases; the other sizes are what
    constructing the assembler and calling it add, on the device and in
    host memory together.  Python object overhead and allocator rounding are
    not counted."""

    kind: str
    rows: int
    columns: int
    entity_count: int
    quadrature_points_per_entity: int
    row_local_dofs: int
    column_local_dofs: int
    nnz_upper_bound: int
    basis_bytes: int
    native_tabulation_bytes: int
    dof_map_bytes: int
    csr_bytes_upper_bound: int
    scatter_bytes: int
    coloring_bytes_upper_bound: int
    pattern_temporary_bytes_upper_bound: int
    staging_bytes_upper_bound: int
    assumptions: tuple = ()

    @property
    def persistent_incremental_bytes_upper_bound(self) -> int:
        return (self.native_tabulation_bytes + self.dof_map_bytes + self.csr_bytes_upper_bound
                + self.scatter_bytes + self.coloring_bytes_upper_bound)

    @property
    def construction_peak_incremental_bytes_upper_bound(self) -> int:
        return (self.persistent_incremental_bytes_upper_bound + self.pattern_temporary_bytes_upper_bound
                + self.staging_bytes_upper_bound)

    @property
    def construction_peak_total_bytes_upper_bound(self) -> int:
        return self.basis_bytes + self.construction_peak_incremental_bytes_upper_bound

    @property
    def largest_incremental_allocation(self):
        items = {
            "native tabulation": self.native_tabulation_bytes,
            "DOF map": self.dof_map_bytes,
            "CSR": self.csr_bytes_upper_bound,
            "element matrices": self.scatter_bytes,
            "row incidence": self.coloring_bytes_upper_bound,
            "temporary CSR pattern": self.pattern_temporary_bytes_upper_bound,
            "coefficient staging": self.staging_bytes_upper_bound,
        }
        return max(items.items(), key=lambda item: item[1])

    def fits_in(self, available_bytes: int, *, safety_factor: float = 1.25) -> bool:
        if available_bytes < 0:
            raise ValueError("available_bytes must be nonnegative")
        if safety_factor < 1.0:
            raise ValueError("safety_factor must be at least 1")
        return self.construction_peak_total_bytes_upper_bound * safety_factor <= available_bytes


class AssemblyMemoryBudgetError(MemoryError):
    """Raised before any device allocation when an estimate exceeds its budget."""

    def __init__(self, estimate, memory_limit_bytes, safety_factor):
        self.estimate = estimate
        self.memory_limit_bytes = memory_limit_bytes
        self.safety_factor = safety_factor
        self.required_bytes = math.ceil(estimate.construction_peak_total_bytes_upper_bound * safety_factor)
        name, size = estimate.largest_incremental_allocation
        self.largest_allocation = name
        self.largest_allocation_bytes = size
        super().__init__(
            "native assembly memory budget exceeded: "
            f"required={format_bytes(self.required_bytes)}, "
            f"estimated_peak={format_bytes(estimate.construction_peak_total_bytes_upper_bound)}, "
            f"budget={format_bytes(memory_limit_bytes)}, safety_factor={safety_factor:.3g}, "
            f"largest={name} ({format_bytes(size)}), rows={estimate.rows}, columns={estimate.columns}, "
            f"entities={estimate.entity_count}, "
            f"local_dofs={estimate.row_local_dofs}x{estimate.column_local_dofs}")


def enforce_memory_budget(estimate, memory_limit_bytes, *, safety_factor=1.25):
    """Validate a budget and raise before any allocation if the estimate does
    not fit (preflight.py:142-158: the safety factor is checked even without
    a budget; a budget must be a positive integer)."""
    if not math.isfinite(safety_factor) or safety_factor < 1.0:
        raise ValueError("memory_safety_factor must be at least 1")
    if memory_limit_bytes is None:
        return
    if isinstance(memory_limit_bytes, (bool, np.bool_)) or not isinstance(memory_limit_bytes, (int, np.integer)):
        raise TypeError("memory_limit_bytes must be an integer or None")
    if memory_limit_bytes <= 0:
        raise ValueError("memory_limit_bytes must be positive")
    if not estimate.fits_in(int(memory_limit_bytes), safety_factor=safety_factor):
        raise AssemblyMemoryBudgetError(estimate, int(memory_limit_bytes), safety_factor)


# ---------------------------------------------------------------- held arrays

def _buffer_key(a):
    """(address, bytes) of a numpy array or torch tensor, else None."""
    if isinstance(a, np.ndarray):
        return (a.__array_interface__["data"][0], int(a.nbytes)) if a.size else None
    if hasattr(a, "data_ptr") and hasattr(a, "nbytes"):
        return (int(a.data_ptr()), int(a.nbytes)) if a.numel() else None
    return None


def _collect(value, out, depth):
    key = _buffer_key(value)
    if key is not None:
        out.add(key)
    elif depth > 0:
        if isinstance(value, dict):
            items = value.values()
        elif isinstance(value, (tuple, list)):
            items = value
        elif is_dataclass(value) and not isinstance(value, type):
            items = [getattr(value, f.name) for f in fields(value)]
        else:
            return
        for item in items:
            _collect(item, out, depth - 1)


# the caller's mesh, and views of its connectivity
_NOT_HELD = frozenset({"mesh", "field_connectivity"})


def held_bytes(*bases):
    """Bytes of the arrays the bases hold, host and device, each buffer
    counted once: attributes that are arrays or tensors (one level into
    dicts, tuples and dataclasses, two into a DOF map's topology) and the
    device copies of each mesh.  Reads attributes only: nothing is made."""
    keys = set()
    for b in bases:
        for name, value in vars(b).items():
            if name not in _NOT_HELD:
                _collect(value, keys, 2)
        _collect(vars(b.mesh).get("_device_cache", {}), keys, 1)
    return sum(size for _, size in keys)


def _validate_basis(basis, label):
    if not all(hasattr(basis, name) for name in ("N", "mesh", "W", "_nodes", "_comp", "element_dofs")):
        raise TypeError(f"{label} is not a nodal tetrahedral Basis of this backend")


def _pattern_bytes(E, Lr, Lc, rows, nnz):
    """(DOF-map copies, CSR, row incidence, temporaries) of one pattern and
    its matrix target, in bytes."""
    tr, tc = E * Lr, E * Lc
    dof_copies = _I32 * (tr + tc)
    csr = (_I32 * (rows + 1) + (_I32 + _F64) * nnz  # device CSR and values
           + 2 * ((_F64 + _I32) * nnz + _I64 * (rows + 1)))  # page-locked host matrix and one copy
    incidence = 20 * tr + _I32 * (rows + 1) + 2 * 8 * rows
    temporary = 128 * (rows + 1) + _I32 * nnz
    return dof_copies, csr, incidence, temporary


def estimate_bilinear_memory(basis, trial_basis=None):
    """Estimate for ``NativeBilinearForm`` / ``NativeTensorForm`` (one basis)
    or ``NativeCrossBilinearForm`` (test ``basis`` and ``trial_basis``),
    computed from sizes alone: no pattern is built and nothing is allocated
    (preflight.py:209-290)."""
    trial = basis if trial_basis is None else trial_basis
    _validate_basis(basis, "test_basis")
    _validate_basis(trial, "trial_basis")
    same = trial is basis
    E, Q = basis.mesh.nelements, len(basis.W)
    if trial.mesh.nelements != E or len(trial.W) != Q:
        raise ValueError("test and trial basis quadrature shapes must match")
    Lr, Lc = basis._nodes * basis._comp, trial._nodes * trial._comp
    rows, columns = int(basis.N), int(trial.N)
    nnz = min(rows * columns, E * Lr * Lc)
    distinct = (basis,) if same else (basis, trial)
    tabulation = sum(E * Q * (4 * b._nodes + 7) * _F64 for b in distinct if getattr(b, "_tab", None) is None)
    if not same:  # the cross form compares the bases' dx and points on the host
        tabulation += sum(4 * E * Q * _F64 for b in distinct if "x" not in getattr(b, "_tab_host", {}))
    dof_maps = sum(E * b._nodes * b._comp * _I32 for b in distinct if not hasattr(b, "_dofs_dev"))
    dof_copies, csr, incidence, temporary = _pattern_bytes(E, Lr, Lc, rows, nnz)
    per_point = (9 if basis._comp == 1 else 4) if same else 9 * basis._comp * trial._comp
    geometry = 16 * _F64 * E if same and basis._comp == 1 else 0
    return AssemblyMemoryEstimate(
        kind="bilinear" if same else "cross-bilinear", rows=rows, columns=columns, entity_count=E,
        quadrature_points_per_entity=Q, row_local_dofs=Lr, column_local_dofs=Lc, nnz_upper_bound=nnz,
        basis_bytes=held_bytes(*distinct), native_tabulation_bytes=tabulation,
        dof_map_bytes=dof_maps + dof_copies, csr_bytes_upper_bound=csr, scatter_bytes=E * Lr * Lc * _F64,
        coloring_bytes_upper_bound=incidence, pattern_temporary_bytes_upper_bound=temporary,
        staging_bytes_upper_bound=geometry + 2 * per_point * E * Q * _F64,
        assumptions=(
            "int32 device DOF maps, CSR offsets and columns; float64 values",
            "CSR nnz is an adjacency-free upper bound, not an exact count",
            "element matrices are float64 (the FP32-pair precisions write as much or less)",
            "per-point coefficients of every kind are staged (page-locked and device copies)",
            "the CUDA sparse tensor of assemble_torch (int64 offsets and columns) is not counted",
            "Python objects and allocator rounding are excluded",
        ))


def estimate_n1_memory(basis, E, Q, rows):
    """Estimate for the Nedelec assembler: 6 x 6 element matrices over the
    edge DOFs; the basis already holds the device edge map, the assembler
    keeps an (E, 6) copy of it for the pattern."""
    nnz = min(rows * rows, E * 36)
    dof_copies, csr, incidence, temporary = _pattern_bytes(E, 6, 6, rows, nnz)
    return AssemblyMemoryEstimate(
        kind="hcurl_tet_n1", rows=rows, columns=rows, entity_count=E, quadrature_points_per_entity=Q,
        row_local_dofs=6, column_local_dofs=6, nnz_upper_bound=nnz, basis_bytes=held_bytes(basis),
        native_tabulation_bytes=0, dof_map_bytes=dof_copies + 6 * E * _I32, csr_bytes_upper_bound=csr,
        scatter_bytes=36 * E * _F64, coloring_bytes_upper_bound=incidence,
        pattern_temporary_bytes_upper_bound=temporary, staging_bytes_upper_bound=3 * E * Q * _F64,
        assumptions=(
            "int32 device DOF maps, CSR offsets and columns; float64 values",
            "CSR nnz is an adjacency-free upper bound, not an exact count",
            "per-point mass and curl coefficients are staged on the device with a unit array",
            "Python objects and allocator rounding are excluded",
        ))
