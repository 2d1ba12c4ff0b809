"""magnus_gb300 — GB300-native Magnus-expansion engine, drop-in for ``magnus``.

Same public surface as s-cavalier/magnus-dp's ``magnus`` package
(src/api/magnus/__init__.py:23-229 and the ``_core`` module of
src/api/pybind.cpp:437-543): ``compute``, ``compute_sc``, ``compute_vjp``,
``compute_sc_vjp``, ``replace_gl_table``, ``max_order`` and the dispatch-name
metadata, with the same op semantics (one / many / sum), integrator names,
shapes, carry layout and error messages.  All arithmetic runs on the GB300
through the C ABI of libmagnus_gb300.so.

Differences from the reference, by design:

* ``matrix_backends()`` adds ``"GB300"``.  Every matrix backend name selects
  the one GPU engine ("Fixed2" keeps its d == 2 validity check); "SpaceCurve"
  data goes through ``compute_sc``.
* ``gl_backend`` names are validated and otherwise ignored: the Gauss-Legendre
  lanes are folded into the engine's algebra ("threadpool" is only valid
  inside a JAX FFI call, as in the reference).
* Extra keyword ``precision``: ``"plain"`` (FP64 everywhere; the parity form)
  or ``"mixed"`` (FP32 per-sample products, FP64 carries and sums).
* ``compute_vjp(vjp_data=...)`` checks the carry's shape exactly like the
  reference and then recomputes what it needs from the chunk checkpoints
  (replaying the forward costs less than reading Q*(n-1)*S*d*d values).
* complex64 / complex128 data run on the engine's real kernels: a complex
  d x d matrix problem as the real 2d x 2d problem on
  [[Re A, -Im A], [Im A, Re A]], complex SpaceCurve data as the real 8 x 8
  problem on the embedding of the quaternion right-multiplication matrix of
  (0, f) (both maps are algebra homomorphisms, so the results are exact up to
  rounding); the VJP is the reference's bilinear one.
"""
from __future__ import annotations

import ctypes
import operator
from typing import Callable

import numpy as np

from . import _lib

__all__ = [
    "max_order",
    "numeric_backends",
    "matrix_backends",
    "integrators",
    "gl_backends",
    "ops",
    "replace_gl_table",
    "compute",
    "compute_sc",
    "compute_vjp",
    "compute_sc_vjp",
]

_MATRIX_BACKENDS = ("Fixed2", "Manual", "Blas", "SpaceCurve", "GB300")
_INTEGRATORS = ("Boole", "Simpson", "Trapezoid", "Riemann")
_GL_BACKENDS = ("threadpool", "openmp", "serial")
_NUMERIC = ("float", "double", "std::complex<float>", "std::complex<double>")
_OPS = ("one", "many", "sum")
_UNRESOLVED = "Could not resolve dispatch name option"
_INVALID = "invalid dispatch option (based on params)"


# ------------------------------------------------------------------ metadata
def max_order() -> int:
    """Largest Gauss-Legendre order in the active table; any n with
    (n + 3) // 2 <= max_order() is supported (pybind.cpp:442-446)."""
    return int(_lib.load().mgb_max_order())


def numeric_backends() -> tuple:
    return _NUMERIC


def matrix_backends() -> tuple:
    return _MATRIX_BACKENDS + ("Auto",)


def integrators() -> tuple:
    return _INTEGRATORS + ("Auto",)


def gl_backends() -> tuple:
    return _GL_BACKENDS + ("Auto",)


def ops() -> tuple:
    return _OPS


def replace_gl_table(max_order: int) -> None:
    """Recompute the process-global Gauss-Legendre table up to ``max_order``
    (src/api/magnus/__init__.py:38-55)."""
    table_order = operator.index(max_order)
    if table_order < 1:
        raise ValueError("max_order must be at least 1")
    total = table_order * (table_order + 1) // 2
    weights = np.empty(total, dtype=np.float64)
    nodes = np.empty(total, dtype=np.float64)
    off = 0
    for order in range(1, table_order + 1):
        x, w = np.polynomial.legendre.leggauss(order)
        nodes[off:off + order] = (x + 1) / 2
        weights[off:off + order] = w / 2
        off += order
    lib = _lib.load()
    _lib.check(lib.mgb_set_gl_table(table_order, weights.ctypes.data, nodes.ctypes.data))


# ------------------------------------------------------------------ helpers
def _op_code(op) -> int:
    try:
        return _lib.OP_CODES[op]
    except (KeyError, TypeError):
        raise ValueError("could not deduce kernel op from str in Magnus::Dispatch::op_from_str(std::string_view)") from None


def _resolve(name, names, auto=True) -> str:
    if auto and name == "Auto":
        return "Auto"
    if name in names:
        return name
    raise ValueError(_UNRESOLVED)


def _integrator_code(name) -> int:
    r = _resolve(name, _INTEGRATORS)
    # Auto picks the first valid integrator: Boole (integration/backends.hpp:53-58).
    return _lib.INTEGRATOR_CODES["Boole" if r == "Auto" else r]


def _check_gl_backend(name) -> None:
    r = _resolve(name, _GL_BACKENDS)
    if r == "threadpool":
        raise ValueError(_INVALID)


def _precision_code(precision) -> int:
    try:
        return _lib.PRECISION_CODES[precision]
    except (KeyError, TypeError):
        raise ValueError(f"precision must be 'plain' or 'mixed', got {precision!r}") from None


def _dtype_code(dtype) -> int:
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        return _lib.DTYPE_F32
    if dtype == np.float64:
        return _lib.DTYPE_F64
    if dtype == np.complex64:
        return _lib.DTYPE_C64
    if dtype == np.complex128:
        return _lib.DTYPE_C128
    raise TypeError("magnus only supports dtypes float32, float64, complex64, and complex128")


def _sample_callable(f: Callable, t0, tf, samples, *, dtype=None, vectorized=True) -> np.ndarray:
    """src/api/magnus/__init__.py:58-70."""
    count = operator.index(samples)
    t = np.linspace(t0, tf, count)
    values = f(t) if vectorized else [f(float(ti)) for ti in t]
    return np.ascontiguousarray(np.asarray(values, dtype=dtype))


def _matrix_input_shape(n, shape):
    """composer/backends.hpp:108-122."""
    if n == 0:
        raise ValueError("n must be at least 1")
    if len(shape) != 3:
        raise ValueError("data must have shape (samples, dim, dim)")
    samples, rows, cols = shape
    if samples < 2:
        raise ValueError("data must contain at least two samples")
    if rows == 0 or cols != rows:
        raise ValueError("data must contain square matrices")
    return samples, rows


def _spacecurve_input_shape(n, shape):
    """composer/backends.hpp:124-137."""
    if n == 0:
        raise ValueError("n must be at least 1")
    if len(shape) != 2:
        raise ValueError("data must have shape (samples, 3)")
    samples, width = shape
    if samples < 2:
        raise ValueError("data must contain at least two samples")
    if width != 3:
        raise ValueError("data must have shape (samples, 3)")
    return samples


def _carry_shape(n, samples, dim):
    return ((n + 3) // 2, n - 1, samples, dim, dim)


def _validate_shape(actual, expected, message):
    if tuple(actual) != tuple(expected):
        raise ValueError(message)


def _n_index(n) -> int:
    n = operator.index(n)
    if n < 0:
        raise TypeError("n must be a non-negative integer")
    return n


# ------------------------------------------------------------------ sampled core
def _compute_matrix(n, data, t0, tf, op, matrix_backend, integrator, gl_backend, record_vjp, precision, checkpoint_K):
    data = np.asarray(data)
    code = _dtype_code(data.dtype)
    n = _n_index(n)
    data = np.ascontiguousarray(data)
    samples, dim = _matrix_input_shape(n, data.shape)
    opc = _op_code(op)
    mb = _resolve(matrix_backend, _MATRIX_BACKENDS)
    integ = _integrator_code(integrator)
    _check_gl_backend(gl_backend)
    if mb == "Fixed2" and dim != 2:
        raise ValueError(_INVALID)
    if mb == "SpaceCurve":
        raise ValueError(_INVALID + ": SpaceCurve data goes through compute_sc on the GB300 engine")
    out_shape = (n, dim, dim) if opc == _lib.OP_MANY else (dim, dim)
    out = np.empty(out_shape, dtype=data.dtype)
    carry = np.zeros(_carry_shape(n, samples, dim), dtype=data.dtype) if record_vjp else None
    prob = _lib.make_problem(kind=_lib.KIND_MATRIX, dtype_code=code, precision=_precision_code(precision), op=opc,
                             integrator=integ, n=n, samples=samples, dim=dim, t0=t0, tf=tf,
                             checkpoint_K=checkpoint_K)
    lib = _lib.load()
    _lib.check(lib.mgb_forward_host(ctypes.byref(prob), data.ctypes.data, out.ctypes.data,
                                    carry.ctypes.data if (carry is not None and carry.size) else None))
    return (out, carry) if record_vjp else out


def _compute_spacecurve(n, data, t0, tf, op, integrator, gl_backend, record_vjp, precision, checkpoint_K):
    data = np.asarray(data)
    code = _dtype_code(data.dtype)
    n = _n_index(n)
    data = np.ascontiguousarray(data)
    samples = _spacecurve_input_shape(n, data.shape)
    opc = _op_code(op)
    integ = _integrator_code(integrator)
    _check_gl_backend(gl_backend)
    out = np.empty((n, 3) if opc == _lib.OP_MANY else (3,), dtype=data.dtype)
    carry = np.zeros(_carry_shape(n, samples, 2), dtype=data.dtype) if record_vjp else None
    prob = _lib.make_problem(kind=_lib.KIND_SPACECURVE, dtype_code=code, precision=_precision_code(precision), op=opc,
                             integrator=integ, n=n, samples=samples, dim=2, t0=t0, tf=tf, checkpoint_K=checkpoint_K)
    lib = _lib.load()
    _lib.check(lib.mgb_forward_host(ctypes.byref(prob), data.ctypes.data, out.ctypes.data,
                                    carry.ctypes.data if (carry is not None and carry.size) else None))
    return (out, carry) if record_vjp else out


def _vjp_matrix(n, data, cotangent, vjp_data, t0, tf, op, matrix_backend, integrator, precision, checkpoint_K):
    data = np.asarray(data)
    code = _dtype_code(data.dtype)
    n = _n_index(n)
    data = np.ascontiguousarray(data)
    samples, dim = _matrix_input_shape(n, data.shape)
    opc = _op_code(op)
    cot = np.ascontiguousarray(np.asarray(cotangent, dtype=data.dtype))
    if opc == _lib.OP_MANY:
        _validate_shape(cot.shape, (n, dim, dim), "many output must have shape (n, dim, dim)")
    else:
        _validate_shape(cot.shape, (dim, dim), "one/sum output must have shape (dim, dim)")
    if vjp_data is not None:
        _validate_shape(np.shape(vjp_data), _carry_shape(n, samples, dim), "VJP data has an invalid shape")
    mb = _resolve(matrix_backend, _MATRIX_BACKENDS)
    integ = _integrator_code(integrator)
    if mb == "Fixed2" and dim != 2:
        raise ValueError(_INVALID)
    if mb == "SpaceCurve":
        raise ValueError(_INVALID + ": SpaceCurve data goes through compute_sc_vjp on the GB300 engine")
    dA = np.empty_like(data)
    prob = _lib.make_problem(kind=_lib.KIND_MATRIX, dtype_code=code, precision=_precision_code(precision), op=opc,
                             integrator=integ, n=n, samples=samples, dim=dim, t0=t0, tf=tf, checkpoint_K=checkpoint_K)
    lib = _lib.load()
    _lib.check(lib.mgb_vjp_host(ctypes.byref(prob), data.ctypes.data, cot.ctypes.data, dA.ctypes.data))
    return dA


def _vjp_spacecurve(n, data, cotangent, vjp_data, t0, tf, op, integrator, precision, checkpoint_K):
    data = np.asarray(data)
    code = _dtype_code(data.dtype)
    n = _n_index(n)
    data = np.ascontiguousarray(data)
    samples = _spacecurve_input_shape(n, data.shape)
    opc = _op_code(op)
    cot = np.ascontiguousarray(np.asarray(cotangent, dtype=data.dtype))
    if opc == _lib.OP_MANY:
        _validate_shape(cot.shape, (n, 3), "many spacecurve output must have shape (n, 3)")
    else:
        _validate_shape(cot.shape, (3,), "one/sum spacecurve output must have shape (3,)")
    if vjp_data is not None:
        _validate_shape(np.shape(vjp_data), _carry_shape(n, samples, 2), "VJP data has an invalid shape")
    integ = _integrator_code(integrator)
    dA = np.empty_like(data)
    prob = _lib.make_problem(kind=_lib.KIND_SPACECURVE, dtype_code=code, precision=_precision_code(precision), op=opc,
                             integrator=integ, n=n, samples=samples, dim=2, t0=t0, tf=tf, checkpoint_K=checkpoint_K)
    lib = _lib.load()
    _lib.check(lib.mgb_vjp_host(ctypes.byref(prob), data.ctypes.data, cot.ctypes.data, dA.ctypes.data))
    return dA


# ------------------------------------------------------------------ public API
def compute(n: int, f: Callable, t0: float, tf: float, samples: int, *, op="sum", dtype=None, vectorized=True,
            matrix_backend="Auto", integrator="Auto", gl_backend="Auto", record_vjp=False, precision="plain",
            checkpoint_K=0):
    """Return the Magnus output and, when requested, its saved forward carry
    (src/api/magnus/__init__.py:88-122)."""
    data = _sample_callable(f, t0, tf, samples, dtype=dtype, vectorized=vectorized)
    return _compute_matrix(n, data, t0, tf, op, matrix_backend, integrator, gl_backend, record_vjp, precision,
                           checkpoint_K)


def compute_sc(n: int, f: Callable, t0: float, tf: float, samples: int, *, op="sum", dtype=None, vectorized=True,
               integrator="Auto", gl_backend="Auto", record_vjp=False, precision="plain", checkpoint_K=0):
    """SpaceCurve form (src/api/magnus/__init__.py:125-157)."""
    data = _sample_callable(f, t0, tf, samples, dtype=dtype, vectorized=vectorized)
    return _compute_spacecurve(n, data, t0, tf, op, integrator, gl_backend, record_vjp, precision, checkpoint_K)


def compute_vjp(n: int, f: Callable, cotangent, t0: float, tf: float, samples: int, *, op="sum", dtype=None,
                vectorized=True, matrix_backend="Auto", integrator="Auto", vjp_data=None, precision="plain",
                checkpoint_K=0):
    """VJP with respect to the sampled matrices (src/api/magnus/__init__.py:160-194)."""
    data = _sample_callable(f, t0, tf, samples, dtype=dtype, vectorized=vectorized)
    return _vjp_matrix(n, data, cotangent, vjp_data, t0, tf, op, matrix_backend, integrator, precision, checkpoint_K)


def compute_sc_vjp(n: int, f: Callable, cotangent, t0: float, tf: float, samples: int, *, op="sum", dtype=None,
                   vectorized=True, integrator="Auto", vjp_data=None, precision="plain", checkpoint_K=0):
    """SpaceCurve VJP (src/api/magnus/__init__.py:197-229)."""
    data = _sample_callable(f, t0, tf, samples, dtype=dtype, vectorized=vectorized)
    return _vjp_spacecurve(n, data, cotangent, vjp_data, t0, tf, op, integrator, precision, checkpoint_K)


# Sampled-array entry points with the reference _core signatures
# (src/api/pybind.cpp:487-543), for callers that sample themselves.
class _Core:
    @staticmethod
    def compute(n, data, t0, tf, op="sum", matrix_backend="Auto", integrator="Auto", gl_backend="Auto",
                record_vjp=False, precision="plain", checkpoint_K=0):
        return _compute_matrix(n, data, t0, tf, op, matrix_backend, integrator, gl_backend, record_vjp, precision,
                               checkpoint_K)

    @staticmethod
    def compute_sc(n, data, t0, tf, op="sum", integrator="Auto", gl_backend="Auto", record_vjp=False,
                   precision="plain", checkpoint_K=0):
        return _compute_spacecurve(n, data, t0, tf, op, integrator, gl_backend, record_vjp, precision, checkpoint_K)

    @staticmethod
    def compute_vjp(n, data, cotangent, vjp_data=None, t0=0.0, tf=1.0, op="sum", matrix_backend="Auto",
                    integrator="Auto", precision="plain", checkpoint_K=0):
        return _vjp_matrix(n, data, cotangent, vjp_data, t0, tf, op, matrix_backend, integrator, precision,
                           checkpoint_K)

    @staticmethod
    def compute_sc_vjp(n, data, cotangent, vjp_data=None, t0=0.0, tf=1.0, op="sum", integrator="Auto",
                       precision="plain", checkpoint_K=0):
        return _vjp_spacecurve(n, data, cotangent, vjp_data, t0, tf, op, integrator, precision, checkpoint_K)


_core = _Core()
