"""Runtime controls mirroring python/skfemntv/runtime.py:12-64.

The GPU backend runs every assembly on the device; the thread count is kept
(and validated exactly as in the reference) so existing callers keep working,
and is reported by ``get_num_threads``.  It does not change GPU execution.
"""
from __future__ import annotations

import os
from contextlib import contextmanager

BACKEND = "skfemntv-gb300"
CAPABILITIES = frozenset({
    "native_backend",
    "gpu_assembly",
    "parallel_basis_geometry",
    "parallel_linear_assembly",
    "parallel_bilinear_assembly",
    "parallel_cross_assembly",
    "deterministic_assembly",
    "split_precision_assembly",
})

_threads = 1


def has_capability(name: str) -> bool:
    return name in CAPABILITIES


def available_num_threads() -> int:
    """Host CPUs this process may run on (its affinity mask where the OS
    reports one, else the machine's CPU count); at least 1."""
    try:
        usable = len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        usable = os.cpu_count() or 1
    return usable if usable > 0 else 1


def get_num_threads() -> int:
    return _threads


def set_num_threads(count: int) -> int:
    global _threads
    if isinstance(count, bool) or not isinstance(count, int) or count < 1:
        raise ValueError("thread count must be a positive integer")
    _threads = min(count, available_num_threads())
    return _threads


@contextmanager
def thread_limit(count: int):
    global _threads
    previous = _threads
    effective = set_num_threads(count)
    try:
        yield effective
    finally:
        _threads = previous
