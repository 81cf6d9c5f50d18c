"""Form front end: ``BilinearForm`` / ``LinearForm`` / ``asm`` and the typed
helpers (python/skfemntv/forms.py:68-112, 667-785, 788-1091;
_form_terms.py, _h1_fields.py, _coefficients.py, _form_parameters.py).

A form function is evaluated once with symbolic trial/test fields and a
parameter namespace ``w``.  Attribute access on ``w`` returns the caller's
keyword arrays (or the quadrature points for ``w.x``); unknown names become
symbolic coefficients resolved from the keywords at assembly time.  The
expression must reduce to a sum of typed terms:

    bilinear: dot(u, v) -> value, ddot|dot(grad u, grad v) -> gradient,
              ddot(sym_grad u, sym_grad v) -> symmetric_gradient,
              div(u) * div(v) -> divergence,
              dot(mul(A, grad u), grad v) -> gradient_tensor
    linear:   dot(f, v) -> value, ddot(G, grad v) -> gradient

each optionally scaled by a number or a coefficient.  ``dot(grad u, grad
v)`` is accepted as well as ``ddot`` (the reference only accepts ``ddot``).
Unsupported expressions raise ``UnsupportedNativeForm``; nothing falls back
to another assembler.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any
from weakref import WeakKeyDictionary

import numpy as np

from .errors import UnsupportedNativeForm

# ---------------------------------------------------------------- coefficients


@dataclass(frozen=True)
class Coefficient:
    """A named form parameter resolved from ``asm`` keywords."""

    name: str

    def __getitem__(self, index):
        if isinstance(index, bool) or not isinstance(index, (int, np.integer)):
            raise ValueError("coefficient component index must be an integer")
        return CoefficientComponent(self.name, int(index))


@dataclass(frozen=True)
class CoefficientComponent:
    name: str
    index: int


def _is_symbolic(v):
    return isinstance(v, (Coefficient, CoefficientComponent))


def _resolve(value, params):
    if isinstance(value, Coefficient):
        name, index = value.name, None
    elif isinstance(value, CoefficientComponent):
        name, index = value.name, value.index
    else:
        return value
    if name not in params:
        raise ValueError(f"missing form parameter {name!r}")
    resolved = params[name]
    if index is None:
        return resolved
    try:
        return np.asarray(resolved)[index]
    except IndexError as error:
        raise ValueError(f"form parameter {name!r} has no component {index}") from error


class QuadratureValue:
    """Numeric form value that keeps typed products (a keyword array or w.x)."""

    __array_priority__ = 1000

    def __init__(self, value, name=None):
        self.value = np.asarray(value)
        self.name = name

    def __array__(self, dtype=None, copy=None):
        return np.asarray(self.value, dtype=dtype)

    def __getitem__(self, key):
        try:
            return QuadratureValue(self.value[key])
        except IndexError as error:
            raise ValueError(f"form parameter {self.name!r} has no component {key}") from error

    def _wrap(self, other, op):
        if isinstance(other, (_Term, _Sum, _Field, _LinearTerm, _LinearSum)):
            return NotImplemented
        o = other.value if isinstance(other, QuadratureValue) else other
        return QuadratureValue(op(self.value, np.asarray(o)))

    def __mul__(self, other):
        if isinstance(other, (_Term, _Sum, _Field, _LinearTerm, _LinearSum)):
            return other.__rmul__(self)
        return self._wrap(other, np.multiply)

    def __rmul__(self, other):
        if isinstance(other, (_Term, _Sum, _Field, _LinearTerm, _LinearSum)):
            return other.__mul__(self)
        return QuadratureValue(np.asarray(other) * self.value)

    def __add__(self, o): return self._wrap(o, np.add)
    def __radd__(self, o): return QuadratureValue(np.asarray(o) + self.value)
    def __sub__(self, o): return self._wrap(o, np.subtract)
    def __rsub__(self, o): return QuadratureValue(np.asarray(o) - self.value)
    def __truediv__(self, o): return self._wrap(o, np.divide)
    def __rtruediv__(self, o): return QuadratureValue(np.asarray(o) / self.value)
    def __pow__(self, o): return QuadratureValue(self.value ** o)
    def __neg__(self): return QuadratureValue(-self.value)

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        vals = [i.value if isinstance(i, QuadratureValue) else i for i in inputs]
        return QuadratureValue(getattr(ufunc, method)(*vals, **kwargs))


class Parameters:
    def __init__(self, values):
        self._values = values

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return self._values.get(name, Coefficient(name))

    def __getitem__(self, name):
        return self._values.get(name, Coefficient(name))


def _coefficient_like(v):
    return _is_symbolic(v) or isinstance(v, (np.ndarray, QuadratureValue)) or np.isscalar(v)


# ---------------------------------------------------------------- typed nodes


@dataclass(frozen=True)
class _Field:
    role: str          # "trial" | "test"
    kind: str          # "value" | "grad" | "symgrad" | "div"
    factor: float = 1.0

    def __mul__(self, other):
        if np.isscalar(other):
            return _Field(self.role, self.kind, self.factor * other)
        if isinstance(other, _Field):
            if self.kind == "div" and other.kind == "div" and self.role != other.role:
                return _Term("divergence", None, self.factor * other.factor)
            if self.kind == "value" and other.kind == "value" and self.role != other.role:
                return _Term("value", None, self.factor * other.factor)
            # cross-basis couplings: div(trial) * test value, div(test) * trial value
            if self.kind == "div" and other.kind == "value" and self.role != other.role:
                kind = "column_divergence" if self.role == "trial" else "row_divergence"
                return _Term(kind, None, self.factor * other.factor)
            if self.kind == "value" and other.kind == "div" and self.role != other.role:
                kind = "column_divergence" if other.role == "trial" else "row_divergence"
                return _Term(kind, None, self.factor * other.factor)
            raise UnsupportedNativeForm("unsupported product of form fields")
        if self.role == "test" and self.kind == "value" and _coefficient_like(other):
            return _LinearTerm("value", _coef(other), self.factor)
        return NotImplemented

    __rmul__ = __mul__

    def __neg__(self):
        return _Field(self.role, self.kind, -self.factor)


@dataclass(frozen=True)
class _TensorGrad:
    role: str
    coefficient: Any
    factor: float = 1.0


def _coef(v):
    if _is_symbolic(v):
        return v
    if isinstance(v, QuadratureValue):
        return v.value
    return np.asarray(v)


@dataclass(frozen=True)
class _Term:
    kind: str
    coefficient: Any = None
    factor: float = 1.0

    def __mul__(self, other):
        if np.isscalar(other):
            return _Term(self.kind, self.coefficient, self.factor * other)
        if _coefficient_like(other):
            if self.coefficient is not None:
                raise UnsupportedNativeForm("multiple bilinear coefficients are not supported")
            return _Term(self.kind, _coef(other), self.factor)
        return NotImplemented

    __rmul__ = __mul__

    def __neg__(self):
        return _Term(self.kind, self.coefficient, -self.factor)

    def __add__(self, other):
        if isinstance(other, _Term):
            return _Sum((self, other))
        if isinstance(other, _Sum):
            return _Sum((self,) + other.terms)
        return NotImplemented

    def __sub__(self, other):
        return self + (-other)


@dataclass(frozen=True)
class _Sum:
    terms: tuple

    def __add__(self, other):
        if isinstance(other, _Term):
            return _Sum(self.terms + (other,))
        if isinstance(other, _Sum):
            return _Sum(self.terms + other.terms)
        return NotImplemented

    __radd__ = __add__

    def __mul__(self, other):
        if np.isscalar(other) or _coefficient_like(other):
            return _Sum(tuple(t * other for t in self.terms))
        return NotImplemented

    __rmul__ = __mul__

    def __neg__(self):
        return _Sum(tuple(-t for t in self.terms))

    def __sub__(self, other):
        return self + (-other)


@dataclass(frozen=True)
class _LinearTerm:
    kind: str
    coefficient: Any
    factor: float = 1.0

    def __mul__(self, other):
        if np.isscalar(other):
            return _LinearTerm(self.kind, self.coefficient, self.factor * other)
        return NotImplemented

    __rmul__ = __mul__

    def __neg__(self):
        return _LinearTerm(self.kind, self.coefficient, -self.factor)

    def __add__(self, other):
        if isinstance(other, _LinearTerm):
            return _LinearSum((self, other))
        if isinstance(other, _LinearSum):
            return _LinearSum((self,) + other.terms)
        return NotImplemented

    def __sub__(self, other):
        return self + (-other)


@dataclass(frozen=True)
class _LinearSum:
    terms: tuple

    def __add__(self, other):
        if isinstance(other, _LinearTerm):
            return _LinearSum(self.terms + (other,))
        if isinstance(other, _LinearSum):
            return _LinearSum(self.terms + other.terms)
        return NotImplemented

    __radd__ = __add__

    def __neg__(self):
        return _LinearSum(tuple(-t for t in self.terms))

    def __sub__(self, other):
        return self + (-other)

    def __mul__(self, other):
        if np.isscalar(other):
            return _LinearSum(tuple(t * other for t in self.terms))
        return NotImplemented

    __rmul__ = __mul__


# ---------------------------------------------------------------- helpers


def grad(value):
    if isinstance(value, _Field) and value.kind == "value":
        return _Field(value.role, "grad", value.factor)
    try:
        return value.grad
    except AttributeError as error:
        raise UnsupportedNativeForm("grad() requires a form field") from error


def sym_grad(value):
    if isinstance(value, _Field) and value.kind == "value":
        return _Field(value.role, "symgrad", value.factor)
    g = grad(value)
    return 0.5 * (g + np.einsum("ij...->ji...", g))


def div(value):
    if isinstance(value, _Field) and value.kind == "value":
        return _Field(value.role, "div", value.factor)
    try:
        return np.einsum("ii...->...", value.grad)
    except AttributeError as error:
        raise UnsupportedNativeForm("div() requires a vector field") from error


def mul(left, right):
    """Coefficient @ trial/test gradient."""
    if isinstance(right, _Field) and right.kind == "grad" and _coefficient_like(left):
        return _TensorGrad(right.role, _coef(left), right.factor)
    raise UnsupportedNativeForm("native mul currently supports coefficient @ trial/test gradient")


def _pair(left, right, kinds):
    return (isinstance(left, _Field) and isinstance(right, _Field) and left.role != right.role
            and left.kind in kinds and right.kind in kinds and left.kind == right.kind)


def dot(left, right):
    if isinstance(left, _TensorGrad) and isinstance(right, _Field) and right.kind == "grad":
        if left.role == right.role:
            raise UnsupportedNativeForm("anisotropic contraction requires trial and test gradients")
        return _Term("gradient_tensor", left.coefficient, left.factor * right.factor)
    if isinstance(right, _TensorGrad) and isinstance(left, _Field) and left.kind == "grad":
        if left.role == right.role:
            raise UnsupportedNativeForm("anisotropic contraction requires trial and test gradients")
        return _Term("gradient_tensor", right.coefficient, left.factor * right.factor)
    if _pair(left, right, ("value",)):
        return _Term("value", None, left.factor * right.factor)
    if _pair(left, right, ("grad",)):
        return _Term("gradient", None, left.factor * right.factor)
    if isinstance(right, _Field) and right.role == "test" and right.kind == "value" and _coefficient_like(left):
        return _LinearTerm("value", _coef(left), right.factor)
    if isinstance(left, _Field) and left.role == "test" and left.kind == "value" and _coefficient_like(right):
        return _LinearTerm("value", _coef(right), left.factor)
    if isinstance(left, (_Field, _TensorGrad)) or isinstance(right, (_Field, _TensorGrad)):
        raise UnsupportedNativeForm("unsupported dot() of form fields")
    return np.einsum("i...,i...->...", np.asarray(left), np.asarray(right))


inner = dot


def ddot(left, right):
    if _pair(left, right, ("grad",)):
        return _Term("gradient", None, left.factor * right.factor)
    if _pair(left, right, ("symgrad",)):
        return _Term("symmetric_gradient", None, left.factor * right.factor)
    if isinstance(right, _Field) and right.role == "test" and right.kind == "grad" and _coefficient_like(left):
        return _LinearTerm("gradient", _coef(left), right.factor)
    if isinstance(left, _Field) and left.role == "test" and left.kind == "grad" and _coefficient_like(right):
        return _LinearTerm("gradient", _coef(right), left.factor)
    if isinstance(left, (_Field, _TensorGrad)) or isinstance(right, (_Field, _TensorGrad)):
        raise UnsupportedNativeForm("unsupported ddot() of form fields")
    return np.einsum("ij...,ij...->...", np.asarray(left), np.asarray(right))


# ---------------------------------------------------------------- forms


class _BilinearForm:
    def __init__(self, function):
        self.function = function
        self._native_cache = WeakKeyDictionary()
        self._tensor_cache = WeakKeyDictionary()
        self._cross_cache = WeakKeyDictionary()

    def assemble(self, *bases, **kwargs):
        return asm(self, *bases, **kwargs)


class _LinearForm:
    def __init__(self, function):
        self.function = function
        self._native_cache = WeakKeyDictionary()

    def assemble(self, *bases, **kwargs):
        return asm(self, *bases, **kwargs)


def BilinearForm(function=None, **kwargs):
    if kwargs or function is None:
        return lambda fn: _BilinearForm(fn)
    return _BilinearForm(function)


def LinearForm(function=None, **kwargs):
    if kwargs or function is None:
        return lambda fn: _LinearForm(fn)
    return _LinearForm(function)


class _LazyX(QuadratureValue):
    """w.x: physical quadrature points (component-first), tabulated on demand."""

    def __init__(self, basis):
        self._basis = basis
        self.name = "x"

    @property
    def value(self):
        return np.moveaxis(self._basis.global_coordinates, -1, 0)


def _trace(form, fields, basis, kwargs, context):
    values = {"x": _LazyX(basis)}
    for name, v in kwargs.items():
        values[name] = v if callable(v) else QuadratureValue(v, name)
    try:
        return form.function(*fields, Parameters(values))
    except (UnsupportedNativeForm, ValueError):
        raise
    except Exception as error:
        raise UnsupportedNativeForm(f"{context} contains an unsupported operation: {error}") from error


def _terms(expr, term, total, message):
    if isinstance(expr, total):
        return expr.terms
    if isinstance(expr, term):
        return (expr,)
    raise UnsupportedNativeForm(message)


def _evaluate(coefficient, kwargs, factor, squeeze=False):
    """The term's coefficient times its factor (_coefficients.py:71-86).  A
    factor of 1 keeps the caller's array, so a broadcast view stays a view.
    ``squeeze`` drops the unit axes of an array of more than two dimensions,
    as the reference does for the scalar coefficients of bilinear terms
    (forms.py:302, 463): (E, Q, 1) or (1, E, Q) then reads as (E, Q).  Tensor
    coefficients keep their axes: squeezed, a (3, 3, E, 1) tensor would lose
    its point axis and fail the shape check."""
    if coefficient is None:
        return float(factor)
    v = np.asarray(_resolve(coefficient, kwargs), dtype=np.float64)
    if factor != 1.0:
        v = factor * v
    if squeeze and v.ndim > 2:
        v = np.squeeze(v)
    return v


def _cross_assemble(form, trial_basis, test_basis, kwargs, memory_limit_bytes, memory_safety_factor):
    """Cross-basis BilinearForm (forms.py:407-486): value, gradient and divergence
    terms between a trial and a test basis on one mesh."""
    from .assembly import NativeCrossBilinearForm

    expr = _trace(form, (_Field("trial", "value"), _Field("test", "value")), test_basis, kwargs,
                  "cross-basis BilinearForm")
    terms = _terms(expr, _Term, _Sum, "cross-basis BilinearForm must reduce to value, gradient, or divergence "
                   "contractions")
    by_trial = form._cross_cache.setdefault(trial_basis, WeakKeyDictionary())
    native = by_trial.get(test_basis)
    if native is None:
        native = NativeCrossBilinearForm(test_basis, trial_basis, memory_limit_bytes=memory_limit_bytes,
                                         memory_safety_factor=memory_safety_factor)
        by_trial[test_basis] = native
    result = None
    for t in terms:
        if t.kind not in ("value", "gradient", "row_divergence", "column_divergence"):
            raise UnsupportedNativeForm(f"unsupported cross-basis term kind {t.kind!r}")
        m = native.assemble(t.kind, _evaluate(t.coefficient, kwargs, t.factor, squeeze=True))
        result = m if result is None else result + m
    return result


def asm(form, *bases, num_threads=None, memory_limit_bytes=None, memory_safety_factor=1.25,
        precision="fp64", **kwargs):
    """Assemble on the GPU (drop-in for skfemntv.asm, forms.py:667-785).

    ``precision``: "fp64" (default) or "split_fp32" (split-precision element
    contraction, FP64 geometry and slot sums; affine H1 paths only).
    """
    if num_threads is not None:
        if isinstance(num_threads, bool) or not isinstance(num_threads, int) or num_threads < 1:
            raise ValueError("num_threads must be a positive integer")
    from .assembly import assemble_bilinear, assemble_linear

    if isinstance(form, _LinearForm):
        if len(bases) != 1:
            raise UnsupportedNativeForm("native LinearForm requires one basis")
        basis = bases[0]
        expr = _trace(form, (_Field("test", "value"),), basis, kwargs, "LinearForm")
        terms = _terms(expr, _LinearTerm, _LinearSum,
                       "native LinearForm must reduce to dot(coefficient, v), "
                       "ddot(coefficient, grad(v)), or a sum of those terms")
        return assemble_linear(form, basis, [(t.kind, _evaluate(t.coefficient, kwargs, t.factor)) for t in terms])
    if isinstance(form, _BilinearForm):
        if len(bases) == 2:
            if num_threads is not None:
                raise UnsupportedNativeForm("per-call threads are not yet supported for cross-basis BilinearForm")
            return _cross_assemble(form, bases[0], bases[1], kwargs, memory_limit_bytes, memory_safety_factor)
        if len(bases) != 1:
            raise UnsupportedNativeForm("native BilinearForm currently requires one shared basis")
        basis = bases[0]
        expr = _trace(form, (_Field("trial", "value"), _Field("test", "value")), basis, kwargs,
                      "BilinearForm")
        terms = _terms(expr, _Term, _Sum,
                       "native BilinearForm must reduce to dot(u, v), ddot(grad(u), grad(v)), "
                       "or a sum of those terms")
        return assemble_bilinear(
            form, basis, [(t.kind, _evaluate(t.coefficient, kwargs, t.factor, squeeze=t.kind != "gradient_tensor"))
                          for t in terms],
            precision=precision, memory_limit_bytes=memory_limit_bytes,
            memory_safety_factor=memory_safety_factor)
    raise TypeError(
        "skfemntv_gb300.asm accepts forms created by skfemntv_gb300.LinearForm or "
        "skfemntv_gb300.BilinearForm; use skfem.asm explicitly for scikit-fem forms")
