"""ctypes binding of libmagnus_gb300.so (the C ABI in include/magnus_gb300.h).

The shared library is built in-tree (``make -C magnus-dp_gb300``, or
``__graft_entry__.build()``) next to this file.  Importing this module on a
machine where the library is missing raises ImportError: there is no CPU
fallback for the engine.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmagnus_gb300.so")

KIND_MATRIX, KIND_SPACECURVE = 0, 1
DTYPE_F32, DTYPE_F64, DTYPE_C64, DTYPE_C128 = 0, 1, 2, 3
PRECISION_PLAIN, PRECISION_MIXED = 0, 1
OP_ONE, OP_MANY, OP_SUM = 0, 1, 2
INTEGRATOR_CODES = {"Boole": 0, "Simpson": 1, "Trapezoid": 2, "Riemann": 3}
OP_CODES = {"one": OP_ONE, "ONE": OP_ONE, "many": OP_MANY, "MANY": OP_MANY, "sum": OP_SUM, "SUM": OP_SUM}
PRECISION_CODES = {"plain": PRECISION_PLAIN, "mixed": PRECISION_MIXED}

OK, ERR_INVALID, ERR_TYPE, ERR_CUDA, ERR_OOM, ERR_TIMEOUT = 0, 1, 2, 3, 4, 5


class MagnusDeviceError(RuntimeError):
    """A CUDA call inside the engine failed or a bounded device wait gave up."""


class Problem(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("op", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("checkpoint_K", ctypes.c_uint32),
        ("n", ctypes.c_uint64),
        ("samples", ctypes.c_uint64),
        ("dim", ctypes.c_uint64),
        ("t0", ctypes.c_double),
        ("tf", ctypes.c_double),
    ]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 40), ("launches", ctypes.c_uint64), ("total_ms", ctypes.c_double),
                ("first_start_ms", ctypes.c_double), ("last_end_ms", ctypes.c_double)]


# name -> (restype, argtypes) for every symbol the header declares
_VP = ctypes.c_void_p
_PP = ctypes.POINTER(Problem)
SIGNATURES = {
    "mgb_forward": (ctypes.c_int, [_PP, _VP, _VP, _VP, _VP, _VP]),
    "mgb_vjp": (ctypes.c_int, [_PP, _VP, _VP, _VP, _VP, _VP]),
    "mgb_checkpoint_bytes": (ctypes.c_size_t, [_PP]),
    "mgb_forward_batched": (ctypes.c_int, [_PP, ctypes.c_size_t, _VP, _VP, _VP, _VP]),
    "mgb_vjp_batched": (ctypes.c_int, [_PP, ctypes.c_size_t, _VP, _VP, _VP, _VP, _VP]),
    "mgb_forward_host": (ctypes.c_int, [_PP, _VP, _VP, _VP]),
    "mgb_vjp_host": (ctypes.c_int, [_PP, _VP, _VP, _VP]),
    "mgb_fwd_vjp_host_batched": (ctypes.c_int, [_PP, ctypes.c_size_t, _VP, _VP, _VP, _VP]),
    "mgb_set_gl_table": (ctypes.c_int, [ctypes.c_size_t, _VP, _VP]),
    "mgb_max_order": (ctypes.c_size_t, []),
    "mgb_device_check": (ctypes.c_int, []),
    "mgb_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_int64, _VP]),
    "mgb_last_error": (ctypes.c_char_p, []),
    "mgb_version": (ctypes.c_int, []),
    "mgb_forward_noalloc": (ctypes.c_int, [_PP, _VP, _VP, _VP]),
    "mgb_plan_create": (ctypes.c_int, [_PP, ctypes.c_size_t, _VP, _VP, _VP, _VP, ctypes.POINTER(ctypes.c_void_p)]),
    "mgb_plan_forward": (ctypes.c_int, [_VP, _VP]),
    "mgb_plan_vjp": (ctypes.c_int, [_VP, _VP]),
    "mgb_plan_bytes": (ctypes.c_size_t, [_VP]),
    "mgb_plan_describe": (ctypes.c_size_t, [_VP, ctypes.c_char_p, ctypes.c_size_t]),
    "mgb_plan_destroy": (ctypes.c_int, [_VP]),
    "mgb_profile_enable": (ctypes.c_int, [ctypes.c_int]),
    "mgb_profile_read": (ctypes.c_size_t, [ctypes.POINTER(KernelTime), ctypes.c_size_t, ctypes.c_int]),
}


def profile_read(reset=True):
    """{name: (launches, total_ms, first_start_ms, last_end_ms)} recorded
    since the last reset (times after the moment timing was switched on)."""
    lib = load()
    buf = (KernelTime * 256)()
    count = lib.mgb_profile_read(buf, 256, int(reset))
    return {buf[i].name.decode(): (int(buf[i].launches), float(buf[i].total_ms), float(buf[i].first_start_ms),
                                   float(buf[i].last_end_ms)) for i in range(min(count, 256))}

_lib = None


def load():
    """Load the engine library (ImportError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"magnus_gb300: engine library not built ({LIB_PATH} missing); run "
            "`make -C magnus-dp_gb300` or __graft_entry__.build()")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    """Raise the reference's exception type for a non-OK status."""
    if status == OK:
        return
    msg = load().mgb_last_error().decode("utf-8", "replace")
    if status == ERR_INVALID:
        raise ValueError(msg)
    if status == ERR_TYPE:
        raise TypeError(msg)
    if status == ERR_OOM:
        raise MemoryError(msg)
    raise MagnusDeviceError(msg)


def make_problem(*, kind, dtype_code, precision, op, integrator, n, samples, dim, t0, tf, checkpoint_K=0) -> Problem:
    return Problem(kind, dtype_code, precision, op, integrator, checkpoint_K, n, samples, dim, float(t0), float(tf))
