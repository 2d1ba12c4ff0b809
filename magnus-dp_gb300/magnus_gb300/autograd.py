"""Differentiable entry point: ``torch.autograd.Function`` over the engine.

``magnus(A, n, t0, tf, ...)`` takes CUDA tensors and returns the Magnus
output on the same device, launched on torch's current stream through the
device C ABI (mgb_forward_batched / mgb_vjp_batched).  The forward stores the
engine's chunk checkpoints (one FP64 state every ``checkpoint_K`` samples,
mgb_checkpoint_bytes per instance); backward replays each chunk from its
checkpoint instead of keeping the reference's full Q*(n-1)*S*d*d carry
(src/graddata.hpp:20-106).

Shapes: matrix kind  A (S, d, d) or batched (B, S, d, d)
        spacecurve   A (S, 3)    or batched (B, S, 3)
Output: (d, d) / (n, d, d) per instance (spacecurve (3,) / (n, 3)), with a
leading B for batched input.  The VJP uses the reference's bilinear pairing.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib

_DTYPES = {torch.float32: _lib.DTYPE_F32, torch.float64: _lib.DTYPE_F64, torch.complex64: _lib.DTYPE_C64,
           torch.complex128: _lib.DTYPE_C128}


def _problems(A, n, t0, tf, op, integrator, precision, kind, checkpoint_K):
    if A.device.type != "cuda":
        raise ValueError("magnus_gb300.autograd expects CUDA tensors")
    if A.dtype not in _DTYPES:
        raise TypeError("magnus only supports dtypes float32, float64, complex64, and complex128")
    batched = A.dim() == (4 if kind == _lib.KIND_MATRIX else 3)
    Ab = A if batched else A.unsqueeze(0)
    if kind == _lib.KIND_MATRIX:
        if Ab.dim() != 4 or Ab.shape[2] != Ab.shape[3]:
            raise ValueError("data must have shape (samples, dim, dim)")
        dim = Ab.shape[2]
    else:
        if Ab.dim() != 3 or Ab.shape[2] != 3:
            raise ValueError("data must have shape (samples, 3)")
        dim = 2
    Ab = Ab.contiguous()
    opc = _lib.OP_CODES.get(op)
    if opc is None:
        raise ValueError("could not deduce kernel op from str in Magnus::Dispatch::op_from_str(std::string_view)")
    integ = _lib.INTEGRATOR_CODES.get("Boole" if integrator == "Auto" else integrator)
    if integ is None:
        raise ValueError("Could not resolve dispatch name option")
    prec = _lib.PRECISION_CODES.get(precision)
    if prec is None:
        raise ValueError("Could not resolve dispatch name option")
    prob = _lib.make_problem(kind=kind, dtype_code=_DTYPES[A.dtype], precision=prec,
                             op=opc, integrator=integ, n=n, samples=Ab.shape[1], dim=dim, t0=t0, tf=tf,
                             checkpoint_K=checkpoint_K)
    return batched, Ab, prob, dim


def _ptr_array(tensors):
    arr = (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])
    return arr


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class MagnusFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, n, t0, tf, op, integrator, precision, kind, checkpoint_K):
        batched, Ab, prob, dim = _problems(A, n, t0, tf, op, integrator, precision, kind, checkpoint_K)
        lib = _lib.load()
        B = Ab.shape[0]
        per_out = ((n,) if prob.op == _lib.OP_MANY else ()) + ((dim, dim) if kind == _lib.KIND_MATRIX else (3,))
        out = torch.empty((B,) + per_out, dtype=A.dtype, device=A.device)
        ck_bytes = lib.mgb_checkpoint_bytes(ctypes.byref(prob))
        if ck_bytes == 0:
            _lib.check(lib.mgb_forward(ctypes.byref(prob), None, None, None, None, None))
        ck = torch.empty((B, ck_bytes), dtype=torch.uint8, device=A.device)
        probs = (_lib.Problem * B)(*([prob] * B))
        As = [Ab[i] for i in range(B)]
        outs = [out[i] for i in range(B)]
        cks = [ck[i] for i in range(B)]
        _lib.check(lib.mgb_forward_batched(probs, B, _ptr_array(As), _ptr_array(outs), _ptr_array(cks), _stream()))
        ctx.save_for_backward(Ab, ck)
        ctx.meta = (batched, prob)
        return out if batched else out[0]

    @staticmethod
    def backward(ctx, grad_out):
        Ab, ck = ctx.saved_tensors
        batched, prob = ctx.meta
        B = Ab.shape[0]
        g = (grad_out if batched else grad_out.unsqueeze(0)).to(Ab.dtype)
        if Ab.is_complex():
            # torch passes and expects conjugate-Wirtinger gradients; the
            # engine's VJP is the bilinear J^T c, so grad_A = conj(J^T conj(g))
            g = g.conj()
        g = g.resolve_conj().contiguous()
        dA = torch.empty_like(Ab)
        lib = _lib.load()
        probs = (_lib.Problem * B)(*([prob] * B))
        _lib.check(lib.mgb_vjp_batched(probs, B, _ptr_array([Ab[i] for i in range(B)]),
                                       _ptr_array([g[i] for i in range(B)]), _ptr_array([ck[i] for i in range(B)]),
                                       _ptr_array([dA[i] for i in range(B)]), _stream()))
        if Ab.is_complex():
            dA = dA.conj().resolve_conj()
        dA = dA if batched else dA[0]
        return dA, None, None, None, None, None, None, None, None


def magnus(A, n, t0=0.0, tf=1.0, *, op="sum", integrator="Auto", precision="plain", checkpoint_K=0):
    """Differentiable Magnus expansion of sampled matrices A (CUDA tensor)."""
    return MagnusFunction.apply(A, int(n), float(t0), float(tf), op, integrator, precision, _lib.KIND_MATRIX,
                                int(checkpoint_K))


def magnus_sc(F, n, t0=0.0, tf=1.0, *, op="sum", integrator="Auto", precision="plain", checkpoint_K=0):
    """Differentiable SpaceCurve Magnus expansion of sampled 3-vectors F."""
    return MagnusFunction.apply(F, int(n), float(t0), float(tf), op, integrator, precision, _lib.KIND_SPACECURVE,
                                int(checkpoint_K))
