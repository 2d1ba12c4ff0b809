"""Batched device entry points and the torch.autograd.Function, through the
C ABI on device buffers."""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import rel
from magnus_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_uneven_batch_matches_per_instance_oracle(cuda):
    import torch
    rng = np.random.default_rng(21)
    specs = [(2, 33, 2, "many"), (3, 65, 4, "sum"), (8, 17, 6, "one"), (16, 129, 3, "sum"), (5, 257, 5, "many"),
             (1, 9, 2, "sum")]
    As, outs, probs, refs = [], [], [], []
    for d, S, n, op in specs:
        A = rng.standard_normal((S, d, d)) / np.sqrt(d)
        As.append(torch.tensor(A, device=cuda))
        shape = (n, d, d) if op == "many" else (d, d)
        outs.append(torch.empty(shape, dtype=torch.float64, device=cuda))
        probs.append(_lib.make_problem(kind=0, dtype_code=1, precision=0, op=_lib.OP_CODES[op], integrator=0, n=n,
                                       samples=S, dim=d, t0=0.0, tf=1.0, checkpoint_K=8))
        refs.append(O.forward(A, n, 0.0, 1.0, op, "Boole"))
    lib = _lib.load()
    P = (_lib.Problem * len(probs))(*probs)
    pa = (ctypes.c_void_p * len(As))(*[a.data_ptr() for a in As])
    po = (ctypes.c_void_p * len(outs))(*[o.data_ptr() for o in outs])
    _lib.check(lib.mgb_forward_batched(P, len(probs), pa, po, None, None))
    torch.cuda.synchronize()
    for o, r in zip(outs, refs):
        assert rel(o.cpu().numpy(), r) <= 1e-12


@pytest.mark.parametrize("precision,tol", [("plain", 1e-12), ("mixed", 1e-6)])
def test_autograd_batched_matches_oracle(precision, tol, cuda):
    import torch
    from magnus_gb300.autograd import magnus
    rng = np.random.default_rng(5)
    B, S, d, n = 3, 97, 4, 5
    A = rng.standard_normal((B, S, d, d)) / np.sqrt(d)
    cot = rng.standard_normal((B, d, d))
    At = torch.tensor(A, device=cuda, requires_grad=True)
    out = magnus(At, n, 0.0, 1.0, op="sum", integrator="Boole", precision=precision, checkpoint_K=16)
    (out * torch.tensor(cot, device=cuda)).sum().backward()
    for b in range(B):
        assert rel(out[b].detach().cpu().numpy(), O.forward(A[b], n, 0.0, 1.0, "sum", "Boole")) <= tol
        assert rel(At.grad[b].cpu().numpy(), O.vjp(A[b], cot[b], n, 0.0, 1.0, "sum", "Boole")) <= tol


def test_autograd_spacecurve_single(cuda):
    import torch
    from magnus_gb300.autograd import magnus_sc
    rng = np.random.default_rng(6)
    F = rng.standard_normal((129, 3))
    cot = rng.standard_normal((6, 3))
    Ft = torch.tensor(F, device=cuda, requires_grad=True)
    out = magnus_sc(Ft, 6, 0.0, 2.0, op="many", integrator="Simpson")
    (out * torch.tensor(cot, device=cuda)).sum().backward()
    assert rel(out.detach().cpu().numpy(), O.forward_sc(F, 6, 0.0, 2.0, "many", "Simpson")) <= 1e-12
    assert rel(Ft.grad.cpu().numpy(), O.vjp_sc(F, cot, 6, 0.0, 2.0, "many", "Simpson")) <= 1e-12


def test_checkpointed_vjp_equals_recompute(cuda):
    """mgb_vjp with the forward's checkpoints == mgb_vjp recomputing them."""
    import torch
    rng = np.random.default_rng(9)
    S, d, n = 257, 8, 5
    A = torch.tensor(rng.standard_normal((S, d, d)) / 3, device=cuda)
    cot = torch.tensor(rng.standard_normal((d, d)), device=cuda)
    prob = _lib.make_problem(kind=0, dtype_code=1, precision=0, op=_lib.OP_SUM, integrator=0, n=n, samples=S, dim=d,
                             t0=0.0, tf=1.0, checkpoint_K=32)
    lib = _lib.load()
    ck = torch.empty(lib.mgb_checkpoint_bytes(ctypes.byref(prob)), dtype=torch.uint8, device=cuda)
    out = torch.empty((d, d), dtype=torch.float64, device=cuda)
    _lib.check(lib.mgb_forward(ctypes.byref(prob), A.data_ptr(), out.data_ptr(), None, ck.data_ptr(), None))
    g1 = torch.empty_like(A)
    g2 = torch.empty_like(A)
    _lib.check(lib.mgb_vjp(ctypes.byref(prob), A.data_ptr(), cot.data_ptr(), ck.data_ptr(), g1.data_ptr(), None))
    _lib.check(lib.mgb_vjp(ctypes.byref(prob), A.data_ptr(), cot.data_ptr(), None, g2.data_ptr(), None))
    torch.cuda.synchronize()
    assert torch.equal(g1, g2)
