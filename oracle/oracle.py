"""ctypes front end of the C oracle — TEST INFRASTRUCTURE ONLY.

Loads ``oracle/_build/libmagnus_oracle.so`` (built by ``oracle/Makefile``)
and exposes the reference's sampled-array entry points with the reference's
shapes (src/api/pybind.cpp:146-355):

* ``forward(A, n, t0, tf, op, integrator, record_vjp)`` -> out or (out, carry)
* ``vjp(A, cot, n, t0, tf, op, integrator, carry=None)`` -> dA
* ``forward_sc`` / ``vjp_sc``: the SpaceCurve forms, padding (S, 3) data to
  (S, 4) with a zero first component and unpadding the outputs exactly as
  composer/backends.hpp:253-357 does.
* ``batch(...)``: many same-shape instances on host threads (CPU baseline).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmagnus_oracle.so")
_lib = None

MATRIX, SPACECURVE = 0, 1
INTEGRATORS = {"Boole": 0, "Simpson": 1, "Trapezoid": 2, "Riemann": 3}
OPS = {"one": 0, "many": 1, "sum": 2}
DIVISIBILITY = {"Boole": 4, "Simpson": 2, "Trapezoid": 2, "Riemann": 1}


def build() -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        lib = ctypes.CDLL(_LIB_PATH)
        sz, dbl, vp, ip = ctypes.c_size_t, ctypes.c_double, ctypes.c_void_p, ctypes.c_int
        for sfx in ("f64", "f32"):
            f = getattr(lib, "mo_forward_" + sfx)
            f.argtypes = [ip, ip, ip, sz, sz, sz, dbl, dbl, sz, vp, vp, vp, vp, vp]
            f.restype = ip
            g = getattr(lib, "mo_vjp_" + sfx)
            g.argtypes = [ip, ip, ip, sz, sz, sz, dbl, dbl, sz, vp, vp, vp, vp, vp, vp]
            g.restype = ip
        lib.mo_batch.argtypes = [ip, ip, ip, ip, ip, sz, sz, sz, dbl, dbl, sz, vp, vp, sz, vp, vp, vp, ip]
        lib.mo_batch.restype = ip
        _lib = lib
    return _lib


def gl_table(order: int):
    """Gauss-Legendre nodes/weights mapped to [0, 1] (util/gen_nodes.py:20-27)."""
    x, w = np.polynomial.legendre.leggauss(order)
    return np.ascontiguousarray(w / 2, dtype=np.float64), np.ascontiguousarray((x + 1) / 2, dtype=np.float64)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(S, n, integrator):
    if n < 1:
        raise ValueError("n must be at least 1")
    if S < 2:
        raise ValueError("data must contain at least two samples")
    if (S - 1) % DIVISIBILITY[integrator]:
        raise ValueError("sample interval count violates integrator divisibility")


def _fwd(kind, A, n, t0, tf, op, integrator, record_vjp):
    A = np.ascontiguousarray(A)
    dtype = A.dtype
    sfx = "f32" if dtype == np.float32 else "f64"
    S = A.shape[0]
    m = 4 if kind == SPACECURVE else A.shape[1] * A.shape[2]
    d = 2 if kind == SPACECURVE else A.shape[1]
    _check(S, n, integrator)
    Q = (n + 3) // 2
    w, x = gl_table(Q)
    nout = n if op == "many" else 1
    out = np.zeros((nout, m), dtype=dtype)
    carry = np.zeros((Q, n - 1, S, m), dtype=dtype) if record_vjp else None
    rc = getattr(_load(), "mo_forward_" + sfx)(
        kind, INTEGRATORS[integrator], OPS[op], n, S, d, float(t0), float(tf), Q,
        _ptr(w), _ptr(x), _ptr(A), _ptr(out), _ptr(carry))
    if rc != 0:
        raise MemoryError("oracle forward failed")
    return out, carry


def forward(A, n, t0=0.0, tf=1.0, op="sum", integrator="Boole", record_vjp=False):
    A = np.asarray(A)
    S, d = A.shape[0], A.shape[1]
    out, carry = _fwd(MATRIX, A, n, t0, tf, op, integrator, record_vjp)
    out = out.reshape((n, d, d) if op == "many" else (d, d))
    if record_vjp:
        return out, carry.reshape(carry.shape[:3] + (d, d))
    return out


def _pad(v):
    v = np.asarray(v)
    p = np.zeros(v.shape[:-1] + (4,), dtype=v.dtype)
    p[..., 1:] = v
    return p


def forward_sc(F, n, t0=0.0, tf=1.0, op="sum", integrator="Boole", record_vjp=False):
    F = np.asarray(F)
    out, carry = _fwd(SPACECURVE, _pad(F), n, t0, tf, op, integrator, record_vjp)
    out = out[:, 1:]
    out = out if op == "many" else out[0]
    if record_vjp:
        return out, carry.reshape(carry.shape[:3] + (2, 2))
    return out


def _vjp(kind, A, cot, n, t0, tf, op, integrator, carry):
    A = np.ascontiguousarray(A)
    dtype = A.dtype
    sfx = "f32" if dtype == np.float32 else "f64"
    S = A.shape[0]
    m = 4 if kind == SPACECURVE else A.shape[1] * A.shape[2]
    d = 2 if kind == SPACECURVE else A.shape[1]
    _check(S, n, integrator)
    Q = (n + 3) // 2
    w, x = gl_table(Q)
    cot = np.ascontiguousarray(cot, dtype=dtype)
    carry = None if carry is None else np.ascontiguousarray(carry, dtype=dtype)
    dA = np.zeros((S, m), dtype=dtype)
    rc = getattr(_load(), "mo_vjp_" + sfx)(
        kind, INTEGRATORS[integrator], OPS[op], n, S, d, float(t0), float(tf), Q,
        _ptr(w), _ptr(x), _ptr(A), _ptr(cot), _ptr(carry), _ptr(dA))
    if rc != 0:
        raise MemoryError("oracle vjp failed")
    return dA


def vjp(A, cot, n, t0=0.0, tf=1.0, op="sum", integrator="Boole", carry=None):
    A = np.asarray(A)
    return _vjp(MATRIX, A, cot, n, t0, tf, op, integrator, carry).reshape(A.shape)


def vjp_sc(F, cot, n, t0=0.0, tf=1.0, op="sum", integrator="Boole", carry=None):
    F = np.asarray(F)
    dA = _vjp(SPACECURVE, _pad(F), _pad(cot), n, t0, tf, op, integrator, carry)
    return dA[:, 1:]


def batch(A, n, t0, tf, op, integrator, *, kind=MATRIX, cot=None, threads=1):
    """Same-shape instances (B, S, ...) on ``threads`` host threads.

    Forward when ``cot`` is None, else the VJP without a carry.  SpaceCurve
    inputs must already be padded to (B, S, 4)."""
    A = np.ascontiguousarray(A)
    B, S = A.shape[0], A.shape[1]
    is_f32 = int(A.dtype == np.float32)
    m = 4 if kind == SPACECURVE else A.shape[2] * A.shape[3]
    d = 2 if kind == SPACECURVE else A.shape[2]
    Q = (n + 3) // 2
    w, x = gl_table(Q)
    nout = n if op == "many" else 1
    if cot is None:
        out = np.zeros((B, nout, m), dtype=A.dtype)
        c = None
    else:
        out = np.zeros((B, S, m), dtype=A.dtype)
        c = np.ascontiguousarray(cot, dtype=A.dtype)
    rc = _load().mo_batch(int(cot is not None), is_f32, kind, INTEGRATORS[integrator], OPS[op], n, S, d,
                          float(t0), float(tf), Q, _ptr(w), _ptr(x), B, _ptr(A), _ptr(c), _ptr(out), int(threads))
    if rc != 0:
        raise MemoryError("oracle batch failed")
    return out
