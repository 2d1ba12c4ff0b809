"""The C-ABI library loads, exports every symbol include/magnus_gb300.h
declares, and applies the reference's validation contract before touching
the GPU (so these run without a device)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from magnus_gb300 import _lib

HEADER = os.path.join(ROOT, "include", "magnus_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(mgb_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_abi():
    names = declared_functions()
    for required in ("mgb_forward", "mgb_vjp", "mgb_forward_batched", "mgb_vjp_batched", "mgb_forward_host",
                     "mgb_vjp_host", "mgb_checkpoint_bytes", "mgb_set_gl_table", "mgb_max_order",
                     "mgb_last_error", "mgb_version"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for name in declared_functions():
        assert hasattr(lib, name), name
    # and the binding knows the signature of each
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def _prob(**kw):
    base = dict(kind=_lib.KIND_MATRIX, dtype_code=_lib.DTYPE_F64, precision=0, op=_lib.OP_SUM, integrator=0, n=4,
                samples=9, dim=2, t0=0.0, tf=1.0)
    base.update(kw)
    return _lib.make_problem(**base)


@pytest.mark.parametrize("kw,msg", [
    (dict(n=0), "n must be at least 1"),
    (dict(samples=1), "at least two samples"),
    (dict(dim=0), "square matrices"),
    (dict(samples=10), "divisibility"),
    (dict(op=7), "deduce kernel op"),
    (dict(integrator=9), "dispatch name"),
    (dict(n=200), "exceeds GL table"),
    (dict(checkpoint_K=6), "multiple of 4"),
])
def test_validation_messages(kw, msg):
    lib = _lib.load()
    p = _prob(**kw)
    x = np.zeros(64)
    st = lib.mgb_forward_host(ctypes.byref(p), x.ctypes.data, x.ctypes.data, None)
    assert st == _lib.ERR_INVALID
    assert msg in lib.mgb_last_error().decode()


def test_dtype_error_is_type_error():
    lib = _lib.load()
    p = _prob(dtype_code=5)
    x = np.zeros(64)
    with pytest.raises(TypeError, match="supports dtypes"):
        _lib.check(lib.mgb_forward_host(ctypes.byref(p), x.ctypes.data, x.ctypes.data, None))


def test_null_buffers_rejected():
    lib = _lib.load()
    p = _prob()
    with pytest.raises(ValueError, match="must not be null"):
        _lib.check(lib.mgb_forward_host(ctypes.byref(p), None, None, None))


def test_checkpoint_bytes():
    lib = _lib.load()
    # C = ceil(8 / 256) = 1 chunk, n*m = 16 -> (2*1+1)*16 doubles
    assert lib.mgb_checkpoint_bytes(ctypes.byref(_prob())) == 3 * 16 * 8
    p = _prob(samples=1025, checkpoint_K=256)  # 4 chunks
    assert lib.mgb_checkpoint_bytes(ctypes.byref(p)) == 9 * 16 * 8
    assert lib.mgb_checkpoint_bytes(ctypes.byref(_prob(n=0))) == 0


def test_default_checkpoint_interval():
    """Default K (checkpoint_K = 0): 256, except 1024 for mixed-form 4-element
    algebras (SpaceCurve, 2 x 2) with at least 65537 samples; read back
    through the checkpoint size (2C + 1) * n * m doubles."""
    lib = _lib.load()

    def chunks(**kw):
        p = _prob(**kw)
        n, m = p.n, 4 if kw.get("kind") == _lib.KIND_SPACECURVE else p.dim * p.dim
        return (lib.mgb_checkpoint_bytes(ctypes.byref(p)) // (8 * n * m) - 1) // 2

    big = 65537
    assert chunks(samples=big, precision=_lib.PRECISION_MIXED, dtype_code=_lib.DTYPE_F32) == 64
    assert chunks(samples=big, precision=_lib.PRECISION_MIXED, dtype_code=_lib.DTYPE_F32,
                  kind=_lib.KIND_SPACECURVE) == 64
    assert chunks(samples=big, precision=_lib.PRECISION_PLAIN) == 256
    assert chunks(samples=big - 4, precision=_lib.PRECISION_MIXED, dtype_code=_lib.DTYPE_F32) == 256
    assert chunks(samples=big, precision=_lib.PRECISION_MIXED, dtype_code=_lib.DTYPE_F32, dim=4) == 256
    assert chunks(samples=big, precision=_lib.PRECISION_MIXED, dtype_code=_lib.DTYPE_F32, checkpoint_K=128) == 512


def test_gl_table_replace_and_max_order():
    import magnus_gb300 as mg
    assert mg.max_order() == 64
    mg.replace_gl_table(80)
    assert mg.max_order() == 80
    mg.replace_gl_table(64)
    assert mg.max_order() == 64
    with pytest.raises(ValueError, match="at least 1"):
        mg.replace_gl_table(0)
