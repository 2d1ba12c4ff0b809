"""mgb_fwd_vjp_host_batched: forward + VJP of a batch from host buffers with
the copies pipelined against the kernels.  Results equal the device entry
points' (several sub-batches, page-locked buffers through the copy kernel)
and the oracle (pageable buffers through cudaMemcpyAsync)."""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import rel
from magnus_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def _probs(specs, precision, dcode):
    return (_lib.Problem * len(specs))(*[
        _lib.make_problem(kind=0, dtype_code=dcode, precision=precision, op=_lib.OP_SUM, integrator=0, n=n,
                          samples=S, dim=d, t0=0.0, tf=1.0) for d, S, n in specs])


def _arr(ptrs):
    return (ctypes.c_void_p * len(ptrs))(*ptrs)


def test_pinned_multi_subbatch_matches_device_path(cuda):
    import torch
    lib = _lib.load()
    specs = [(32, 4097, 4)] * 36 + [(16, 2049, 5)] * 4  # ~0.6 GB of input: three sub-batches
    rng = np.random.default_rng(5)
    A_h = [torch.tensor(workloads.config0_samples(seed=k, d=d, samples=S).astype(np.float32)).pin_memory()
           for k, (d, S, n) in enumerate(specs)]
    cot_h = [torch.tensor(rng.standard_normal((d, d)).astype(np.float32)).pin_memory() for d, S, n in specs]
    out_h = [torch.empty((d, d), dtype=torch.float32).pin_memory() for d, S, n in specs]
    dA_h = [torch.empty_like(a).pin_memory() for a in A_h]
    probs = _probs(specs, _lib.PRECISION_MIXED, _lib.DTYPE_F32)
    _lib.check(lib.mgb_fwd_vjp_host_batched(probs, len(specs), _arr([t.data_ptr() for t in A_h]),
                                            _arr([t.data_ptr() for t in cot_h]), _arr([t.data_ptr() for t in out_h]),
                                            _arr([t.data_ptr() for t in dA_h])))
    # the same through the device entry points
    A_d = [a.to(cuda) for a in A_h]
    cot_d = [c.to(cuda) for c in cot_h]
    out_d = [torch.empty_like(o, device=cuda) for o in out_h]
    dA_d = [torch.empty_like(a) for a in A_d]
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.mgb_forward_batched(probs, len(specs), _arr([t.data_ptr() for t in A_d]),
                                       _arr([t.data_ptr() for t in out_d]), None, s))
    _lib.check(lib.mgb_vjp_batched(probs, len(specs), _arr([t.data_ptr() for t in A_d]),
                                   _arr([t.data_ptr() for t in cot_d]), None, _arr([t.data_ptr() for t in dA_d]), s))
    torch.cuda.synchronize()
    for k in range(len(specs)):
        assert rel(out_h[k].numpy(), out_d[k].cpu().numpy()) <= 1e-6, k
        assert rel(dA_h[k].numpy(), dA_d[k].cpu().numpy()) <= 1e-6, k
    # and the oracle on two of them
    for k in (0, len(specs) - 1):
        d, S, n = specs[k]
        A64 = A_h[k].numpy().astype(np.float64)
        assert rel(out_h[k].numpy(), O.forward(A64, n, 0.0, 1.0, "sum", "Boole")) <= 1e-6
        assert rel(dA_h[k].numpy(), O.vjp(A64, cot_h[k].numpy().astype(np.float64), n, 0.0, 1.0, "sum",
                                          "Boole")) <= 1e-6


def test_pageable_plain_matches_oracle(cuda):
    lib = _lib.load()
    specs = [(4, 513, 4), (8, 257, 3), (3, 129, 5)]
    rng = np.random.default_rng(9)
    A = [workloads.config0_samples(seed=k, d=d, samples=S) for k, (d, S, n) in enumerate(specs)]
    cot = [rng.standard_normal((d, d)) for d, S, n in specs]
    out = [np.empty((d, d)) for d, S, n in specs]
    dA = [np.empty_like(a) for a in A]
    probs = _probs(specs, _lib.PRECISION_PLAIN, _lib.DTYPE_F64)
    _lib.check(lib.mgb_fwd_vjp_host_batched(probs, len(specs), _arr([a.ctypes.data for a in A]),
                                            _arr([c.ctypes.data for c in cot]), _arr([o.ctypes.data for o in out]),
                                            _arr([g.ctypes.data for g in dA])))
    for (d, S, n), a, c, o, g in zip(specs, A, cot, out, dA):
        assert rel(o, O.forward(a, n, 0.0, 1.0, "sum", "Boole")) <= 1e-12
        assert rel(g, O.vjp(a, c, n, 0.0, 1.0, "sum", "Boole")) <= 1e-12


def test_rejects_null_buffers(cuda):
    lib = _lib.load()
    probs = _probs([(2, 129, 3)], _lib.PRECISION_PLAIN, _lib.DTYPE_F64)
    st = lib.mgb_fwd_vjp_host_batched(probs, 1, _arr([None]), _arr([None]), _arr([None]), _arr([None]))
    assert st == 1 and b"must not be null" in lib.mgb_last_error()


def test_profile_timeline_of_the_pipeline(cuda):
    """With timing on, each sub-batch's stages are recorded as h2d.<b>,
    comp.<b>, d2h.<b> with start and end times: every stage starts after the
    one it depends on has ended (copy in -> kernels -> copy out)."""
    import torch
    lib = _lib.load()
    specs = [(32, 4097, 4)] * 36  # ~0.6 GB of input: more than one sub-batch
    A_h = [torch.tensor(workloads.config0_samples(seed=k, d=d, samples=S).astype(np.float32)).pin_memory()
           for k, (d, S, n) in enumerate(specs)]
    cot_h = [torch.ones((d, d), dtype=torch.float32).pin_memory() for d, S, n in specs]
    out_h = [torch.empty((d, d), dtype=torch.float32).pin_memory() for d, S, n in specs]
    dA_h = [torch.empty_like(a).pin_memory() for a in A_h]
    probs = _probs(specs, _lib.PRECISION_MIXED, _lib.DTYPE_F32)
    args = (probs, len(specs), _arr([t.data_ptr() for t in A_h]), _arr([t.data_ptr() for t in cot_h]),
            _arr([t.data_ptr() for t in out_h]), _arr([t.data_ptr() for t in dA_h]))
    _lib.check(lib.mgb_fwd_vjp_host_batched(*args))
    lib.mgb_profile_enable(1)
    _lib.profile_read(reset=True)
    try:
        _lib.check(lib.mgb_fwd_vjp_host_batched(*args))
    finally:
        lib.mgb_profile_enable(0)
    rec = _lib.profile_read(reset=True)
    subs = sorted(int(k.split(".")[1]) for k in rec if k.startswith("comp."))
    assert len(subs) >= 2, sorted(rec)
    eps = 1e-3  # ms
    for b in subs:
        h, c, o = rec[f"h2d.{b}"], rec[f"comp.{b}"], rec[f"d2h.{b}"]
        for launches, total, start, end in (h, c, o):
            assert launches == 1 and end >= start and abs((end - start) - total) <= 1e-2 * max(total, 1.0)
        assert c[2] >= h[3] - eps and o[2] >= c[3] - eps, (b, h, c, o)
    assert any(k.startswith("chunk") for k in rec), sorted(rec)
