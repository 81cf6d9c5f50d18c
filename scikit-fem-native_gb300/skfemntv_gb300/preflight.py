"""Allocation-free memory estimates and budgets (python/skfemntv/preflight.py
:18-352), restated for the GPU backend: the estimate counts the device
memory an assembler keeps (pattern, incidence lists, DOF map, values, the
per-element scratch of the affine path) and the host CSR it returns."""
from __future__ import annotations

import math
from dataclasses import dataclass


def format_bytes(count: int) -> str:
    value = float(count)
    for unit in ("B", "KiB", "MiB", "GiB", "TiB"):
        if value < 1024.0 or unit == "TiB":
            return f"{value:.1f} {unit}"
        value /= 1024.0
    raise AssertionError("unreachable")


@dataclass(frozen=True)
class AssemblyMemoryEstimate:
    kind: str
    rows: int
    columns: int
    entity_count: int
    quadrature_points_per_entity: int
    row_local_dofs: int
    column_local_dofs: int
    nnz_upper_bound: int
    device_pattern_bytes: int
    device_values_bytes: int
    device_scratch_bytes: int
    host_csr_bytes: int
    pattern_temporary_bytes_upper_bound: int

    @property
    def construction_peak_total_bytes_upper_bound(self) -> int:
        return (self.device_pattern_bytes + self.device_values_bytes + self.device_scratch_bytes
                + self.host_csr_bytes + self.pattern_temporary_bytes_upper_bound)

    @property
    def largest_incremental_allocation(self):
        items = {
            "device pattern": self.device_pattern_bytes,
            "device values": self.device_values_bytes,
            "device scratch": self.device_scratch_bytes,
            "host CSR": self.host_csr_bytes,
            "temporary pattern": self.pattern_temporary_bytes_upper_bound,
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
    if memory_limit_bytes is None:
        return
    if isinstance(memory_limit_bytes, bool) or not isinstance(memory_limit_bytes, int) or memory_limit_bytes < 0:
        raise ValueError("memory_limit_bytes must be a nonnegative integer")
    if not math.isfinite(safety_factor) or safety_factor < 1.0:
        raise ValueError("memory_safety_factor must be a finite value >= 1")
    if not estimate.fits_in(memory_limit_bytes, safety_factor=safety_factor):
        raise AssemblyMemoryBudgetError(estimate, memory_limit_bytes, safety_factor)


def estimate_bilinear_memory(basis, trial_basis=None):
    trial = basis if trial_basis is None else trial_basis
    E = basis.mesh.nelements
    Q = len(basis.W)
    Lr = basis._nodes * basis._comp
    Lc = trial._nodes * trial._comp
    nnz = min(basis.N * trial.N, E * Lr * Lc)
    pattern = 4 * (E * Lr + E * Lc) + 4 * (2 * (basis.N + 1)) + 4 * E * Lr + 4 * nnz
    return AssemblyMemoryEstimate(
        kind="bilinear", rows=basis.N, columns=trial.N, entity_count=E, quadrature_points_per_entity=Q,
        row_local_dofs=Lr, column_local_dofs=Lc, nnz_upper_bound=nnz, device_pattern_bytes=pattern,
        device_values_bytes=8 * nnz, device_scratch_bytes=8 * 16 * E, host_csr_bytes=8 * nnz + 4 * nnz
        + 8 * (basis.N + 1), pattern_temporary_bytes_upper_bound=8 * (basis.N + 1) + 16 * E * Lr)
