"""mgb_forward_noalloc: the forward entry point that allocates no device memory.

It exists for callers that cannot call cudaMalloc while they run — an XLA /
JAX custom call or a framework whose caching allocator already holds the
GPU's memory, or a host that must not allocate or synchronize mid-run.  It
takes its working memory from a fixed array compiled into the library
instead.  These tests call it through the C ABI on device buffers and compare
it with the regular mgb_forward, twice in a row (the array is shared and
keeps the previous call's contents), and check that an oversize problem is
refused with a clear message.  The file is named so that pytest collects it
last; it needs nothing from the other test files.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel
from magnus_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def _problem(kind, dtype_code, precision, op, integrator, n, S, d, K=0):
    return _lib.make_problem(kind=kind, dtype_code=dtype_code, precision=precision, op=op, integrator=integrator,
                             n=n, samples=S, dim=d, t0=0.0, tf=1.0, checkpoint_K=K)


CASES = [
    # (label, kind, torch dtype name, precision, op, integrator, n, S, d, tolerance)
    ("plain-f64-d8-many", _lib.KIND_MATRIX, "float64", _lib.PRECISION_PLAIN, _lib.OP_MANY, 0, 4, 1025, 8, 1e-12),
    ("mixed-f32-d32-sum", _lib.KIND_MATRIX, "float32", _lib.PRECISION_MIXED, _lib.OP_SUM, 0, 5, 2049, 32, 1e-6),
    ("plain-f64-spacecurve", _lib.KIND_SPACECURVE, "float64", _lib.PRECISION_PLAIN, _lib.OP_MANY, 1, 6, 1025, 2,
     1e-12),
    # one thread per chunk (2 x 2 and SpaceCurve data) in FP32
    ("mixed-f32-d2-many", _lib.KIND_MATRIX, "float32", _lib.PRECISION_MIXED, _lib.OP_MANY, 0, 5, 4097, 2, 1e-6),
    ("mixed-f32-spacecurve", _lib.KIND_SPACECURVE, "float32", _lib.PRECISION_MIXED, _lib.OP_MANY, 1, 6, 4097, 2,
     1e-6),
    # the tensor-core kernel at d = 64: one 256-sample chunk slot takes half
    # of the array, so the grid is cut to the single slot that fits
    ("mixed-f32-d64-sum-one-slot", _lib.KIND_MATRIX, "float32", _lib.PRECISION_MIXED, _lib.OP_SUM, 0, 4, 1025, 64,
     1e-6),
    # n = 7: five Gauss-Legendre nodes
    ("plain-f64-d4-n7-trapezoid", _lib.KIND_MATRIX, "float64", _lib.PRECISION_PLAIN, _lib.OP_ONE, 2, 7, 1025, 4,
     1e-12),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_forward_matches_forward_twice(case, cuda):
    import torch
    label, kind, tname, precision, op, integ, n, S, d, tol = case
    tdtype = getattr(torch, tname)
    if kind == _lib.KIND_MATRIX:
        A = torch.tensor(workloads.config0_samples(seed=3, d=d, samples=S), dtype=tdtype, device=cuda)
        out_shape = (n, d, d) if op == _lib.OP_MANY else (d, d)
    else:
        F = workloads.config1_samples_np(*workloads.config1_coeffs(seed=5, batch=1), samples=S, dtype=np.float64)[0]
        A = torch.tensor(F, dtype=tdtype, device=cuda)
        out_shape = (n, 3) if op == _lib.OP_MANY else (3,)
    dcode = _lib.DTYPE_F64 if tname == "float64" else _lib.DTYPE_F32
    prob = _problem(kind, dcode, precision, op, integ, n, S, d)
    lib = _lib.load()
    ref = torch.empty(out_shape, dtype=tdtype, device=cuda)
    _lib.check(lib.mgb_forward(ctypes.byref(prob), A.data_ptr(), ref.data_ptr(), None, None, None))
    torch.cuda.synchronize()
    for _ in range(2):
        out = torch.full(out_shape, float("nan"), dtype=tdtype, device=cuda)
        _lib.check(lib.mgb_forward_noalloc(ctypes.byref(prob), A.data_ptr(), out.data_ptr(), None))
        torch.cuda.synchronize()
        assert rel(out.cpu().numpy(), ref.cpu().numpy()) <= tol


def test_noalloc_refuses_oversize_problem(cuda):
    lib = _lib.load()
    prob = _problem(_lib.KIND_MATRIX, _lib.DTYPE_F64, _lib.PRECISION_PLAIN, _lib.OP_SUM, 0, 6, 65537, 64)
    x = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    with pytest.raises(ValueError, match="MGB_NOALLOC_SCRATCH_BYTES"):
        _lib.check(lib.mgb_forward_noalloc(ctypes.byref(prob), x, x, None))
