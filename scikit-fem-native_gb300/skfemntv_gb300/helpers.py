"""Form helpers (python/skfemntv/helpers.py)."""
import numpy as np

from .forms import ddot, div, dot, grad, inner, mul, sym_grad  # noqa: F401


def trace(value):
    return np.einsum("ii...->...", value)


def transpose(value):
    return np.einsum("ij...->ji...", value)
