"""Autotuner: every launch variant of every chunk-kernel family gives the
oracle's results (forced with MGB_FORCE_VARIANT), and a plan reports the
variant it chose and the times it measured (mgb_plan_describe)."""
import ctypes
import json

import numpy as np
import pytest

import oracle as O
from conftest import rel
from magnus_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def _run_plan(cuda, specs, precision, dtype_name, integrator=0, K=32):
    """Plan forward + VJP over `specs` [(d, S, n)]; returns host data,
    outputs, dA and the plan's description."""
    import torch
    tdtype = getattr(torch, dtype_name)
    dcode = _lib.DTYPE_F64 if dtype_name == "float64" else _lib.DTYPE_F32
    rng = np.random.default_rng(7)
    host, As, outs, cots, dAs, probs = [], [], [], [], [], []
    for k, (d, S, n) in enumerate(specs):
        A = workloads.config0_samples(seed=d + k, d=d, samples=S)
        A = A.astype(np.float64 if dtype_name == "float64" else np.float32)
        cot = rng.standard_normal((d, d)).astype(A.dtype)
        host.append((A, cot, n))
        As.append(torch.tensor(A, device=cuda))
        outs.append(torch.empty((d, d), dtype=tdtype, device=cuda))
        cots.append(torch.tensor(cot, device=cuda))
        dAs.append(torch.empty_like(As[-1]))
        probs.append(_lib.make_problem(kind=0, dtype_code=dcode, precision=precision, op=_lib.OP_SUM,
                                       integrator=integrator, n=n, samples=S, dim=d, t0=0.0, tf=1.0, checkpoint_K=K))
    lib = _lib.load()
    ptrs = lambda ts: (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])  # noqa: E731
    P = (_lib.Problem * len(probs))(*probs)
    plan = ctypes.c_void_p()
    _lib.check(lib.mgb_plan_create(P, len(probs), ptrs(As), ptrs(outs), ptrs(cots), ptrs(dAs), ctypes.byref(plan)))
    try:
        need = lib.mgb_plan_describe(plan, None, 0)
        buf = ctypes.create_string_buffer(need)
        lib.mgb_plan_describe(plan, buf, need)
        desc = json.loads(buf.value.decode())
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.check(lib.mgb_plan_forward(plan, stream))
        _lib.check(lib.mgb_plan_vjp(plan, stream))
        torch.cuda.synchronize()
        _lib.check(lib.mgb_device_check())
    finally:
        _lib.check(lib.mgb_plan_destroy(plan))
    return host, [o.cpu().numpy() for o in outs], [g.cpu().numpy() for g in dAs], desc


RULES = {0: "Boole", 1: "Simpson", 2: "Trapezoid", 3: "Riemann"}


@pytest.mark.parametrize("d,nvariants,precision,dtype_name,tol,kernel", [
    # 2: tcgen05 forward + warp-MMA VJP, 3: warp-MMA forward and VJP
    (32, 4, _lib.PRECISION_MIXED, "float32", 1e-6, ["k_tile", "k_tile", "k_tiletc", "k_mma32"]),
    (16, 2, _lib.PRECISION_MIXED, "float32", 1e-6, "k_tile"),
    (64, 5, _lib.PRECISION_MIXED, "float32", 1e-6, "k_bigtc"),  # 4: one accumulator pair, 3 CTAs/SM
    (128, 3, _lib.PRECISION_MIXED, "float32", 1e-6, "k_bigtc"),  # 2: one accumulator pair, 2 CTAs/SM
    (8, 3, _lib.PRECISION_PLAIN, "float64", 1e-12, "k_chunk"),
])
@pytest.mark.parametrize("integrator", [0, 1, 2, 3])
def test_every_variant_matches_oracle(d, nvariants, precision, dtype_name, tol, kernel, integrator, cuda, monkeypatch):
    S = {0: 129, 1: 131, 2: 97, 3: 90}[integrator]
    specs = [(d, S, 4), (d, 2 * S - 1, 3)]
    for v in range(nvariants):
        monkeypatch.setenv("MGB_FORCE_VARIANT", str(v))
        host, outs, dAs, desc = _run_plan(cuda, specs, precision, dtype_name, integrator=integrator)
        seg = desc["segments"][0]
        want = kernel[v] if isinstance(kernel, list) else kernel
        assert seg["kernel"] == want and seg["variant"] == v, seg
        for (A, cot, n), o, g in zip(host, outs, dAs):
            A64 = A.astype(np.float64)
            ref = O.forward(A64, n, 0.0, 1.0, "sum", RULES[integrator])
            gref = O.vjp(A64, cot.astype(np.float64), n, 0.0, 1.0, "sum", RULES[integrator])
            assert rel(o, ref) <= tol, (v, rel(o, ref))
            assert rel(g, gref) <= tol, (v, rel(g, gref))


def test_plan_reports_tuned_variant(cuda, monkeypatch):
    monkeypatch.delenv("MGB_FORCE_VARIANT", raising=False)
    monkeypatch.setenv("MGB_AUTOTUNE", "1")
    specs = [(32, 1025, 5)] * 4 + [(64, 513, 4)] * 2
    host, outs, dAs, desc = _run_plan(cuda, specs, _lib.PRECISION_MIXED, "float32", K=64)
    by_d = {s["d"]: s for s in desc["segments"]}
    assert by_d[32]["kernel"] in ("k_tile", "k_tiletc", "k_mma32") and by_d[64]["kernel"] == "k_bigtc"
    for seg, nv in ((by_d[32], 4), (by_d[64], 5)):
        ms = seg["tuned_ms"]
        assert len(ms) == nv and all(t > 0 for t in ms), seg
        assert ms[seg["variant"]] == min(ms), seg  # the fastest (ties: either)
    for (A, cot, n), o in zip(host, outs):
        assert rel(o, O.forward(A.astype(np.float64), n, 0.0, 1.0, "sum", "Boole")) <= 1e-6


def test_autotune_off_keeps_variant_zero(cuda, monkeypatch):
    monkeypatch.delenv("MGB_FORCE_VARIANT", raising=False)
    monkeypatch.setenv("MGB_AUTOTUNE", "0")
    _, _, _, desc = _run_plan(cuda, [(16, 257, 4)], _lib.PRECISION_MIXED, "float32")
    seg = desc["segments"][0]
    assert seg["variant"] == 0 and seg["tuned_ms"] == []


@pytest.mark.parametrize("precision,dtype_name,tol", [(_lib.PRECISION_MIXED, "float32", 1e-6),
                                                      (_lib.PRECISION_PLAIN, "float64", 1e-12)])
def test_scratch_cut_keeps_results(precision, dtype_name, tol, cuda, monkeypatch):
    """A scratch budget below the segments' asks shrinks every segment's slot
    count in the same proportion; the thread-per-chunk kernel (d = 2) then
    runs with a slot count that is not a multiple of its block size, and its
    last block's spare threads must stay off the scratch."""
    monkeypatch.setenv("MGB_SCRATCH_MB", "1")
    specs = [(2, 4097, 4)] * 6 + [(64, 257, 4)]
    host, outs, dAs, desc = _run_plan(cuda, specs, precision, dtype_name, K=8)
    seg = next(s for s in desc["segments"] if s["d"] == 2)
    assert seg["slots"] < seg["chunks"] and seg["slots"] % 128 != 0, seg
    for (A, cot, n), o, g in zip(host, outs, dAs):
        A64 = A.astype(np.float64)
        assert rel(o, O.forward(A64, n, 0.0, 1.0, "sum", "Boole")) <= tol
        assert rel(g, O.vjp(A64, cot.astype(np.float64), n, 0.0, 1.0, "sum", "Boole")) <= tol
