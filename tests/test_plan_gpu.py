"""Plans (mgb_plan_*): an uneven batch split into per-dimension segments,
and a forward + VJP captured once into a CUDA graph and replayed."""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import rel
from magnus_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def _make(cuda, specs, precision, dtype_name, seed=0):
    import torch
    tdtype = getattr(torch, dtype_name)
    dcode = _lib.DTYPE_F64 if dtype_name == "float64" else _lib.DTYPE_F32
    rng = np.random.default_rng(seed)
    As, outs, cots, dAs, probs, host = [], [], [], [], [], []
    for k, (d, S, n) in enumerate(specs):
        A = workloads.config0_samples(seed=seed + k, d=d, samples=S)
        if dtype_name == "float32":
            A = A.astype(np.float32)
        cot = rng.standard_normal((d, d)).astype(A.dtype)
        host.append((A, cot, n))
        As.append(torch.tensor(A, device=cuda))
        outs.append(torch.empty((d, d), dtype=tdtype, device=cuda))
        cots.append(torch.tensor(cot, device=cuda))
        dAs.append(torch.empty_like(As[-1]))
        probs.append(_lib.make_problem(kind=0, dtype_code=dcode, precision=precision, op=_lib.OP_SUM, integrator=0,
                                       n=n, samples=S, dim=d, t0=0.0, tf=1.0, checkpoint_K=64))
    return As, outs, cots, dAs, probs, host


def _ptrs(ts):
    return (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])


SPECS = [(2, 129, 3), (32, 257, 5), (8, 97, 4), (16, 161, 2), (32, 129, 4), (4, 65, 6), (16, 513, 5), (3, 33, 3)]


@pytest.mark.parametrize("precision,dtype_name,tol", [(_lib.PRECISION_PLAIN, "float64", 1e-12),
                                                      (_lib.PRECISION_MIXED, "float32", 2e-6)])
def test_plan_uneven_batch(precision, dtype_name, tol, cuda):
    import torch
    As, outs, cots, dAs, probs, host = _make(cuda, SPECS, precision, dtype_name)
    lib = _lib.load()
    P = (_lib.Problem * len(probs))(*probs)
    plan = ctypes.c_void_p()
    _lib.check(lib.mgb_plan_create(P, len(probs), _ptrs(As), _ptrs(outs), _ptrs(cots), _ptrs(dAs), ctypes.byref(plan)))
    try:
        assert lib.mgb_plan_bytes(plan) > 0
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.check(lib.mgb_plan_forward(plan, stream))
        _lib.check(lib.mgb_plan_vjp(plan, stream))
        torch.cuda.synchronize()
    finally:
        _lib.check(lib.mgb_plan_destroy(plan))
    for (A, cot, n), o, g in zip(host, outs, dAs):
        A64 = A.astype(np.float64)
        assert rel(o.cpu().numpy(), O.forward(A64, n, 0.0, 1.0, "sum", "Boole")) <= tol
        assert rel(g.cpu().numpy(), O.vjp(A64, cot.astype(np.float64), n, 0.0, 1.0, "sum", "Boole")) <= tol


def test_plan_cuda_graph_capture_and_replay(cuda):
    import torch
    As, outs, cots, dAs, probs, host = _make(cuda, SPECS[:5], _lib.PRECISION_MIXED, "float32", seed=3)
    lib = _lib.load()
    P = (_lib.Problem * len(probs))(*probs)
    plan = ctypes.c_void_p()
    _lib.check(lib.mgb_plan_create(P, len(probs), _ptrs(As), _ptrs(outs), _ptrs(cots), _ptrs(dAs), ctypes.byref(plan)))
    try:
        # eager reference run
        s0 = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.check(lib.mgb_plan_forward(plan, s0))
        _lib.check(lib.mgb_plan_vjp(plan, s0))
        torch.cuda.synchronize()
        ref_out = [o.clone() for o in outs]
        ref_dA = [g.clone() for g in dAs]
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            _lib.check(lib.mgb_plan_forward(plan, s))
            _lib.check(lib.mgb_plan_vjp(plan, s))
        for _ in range(2):
            for o in outs:
                o.fill_(float("nan"))
            for d in dAs:
                d.fill_(float("nan"))
            g.replay()
            torch.cuda.synchronize()
            for o, r in zip(outs, ref_out):
                assert torch.equal(o, r)
            for d, r in zip(dAs, ref_dA):
                assert torch.equal(d, r)
        del g
    finally:
        _lib.check(lib.mgb_plan_destroy(plan))
