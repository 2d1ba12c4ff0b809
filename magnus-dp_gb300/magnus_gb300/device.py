"""Device-side sampling and the consumer step.

The reference samples f(t) on the host (numpy, src/api/magnus/__init__.py:
58-70) and its benchmarks exponentiate Omega with scipy
(tests/bench.py:89-93).  Here f is a torch callable evaluated on a CUDA
tensor of sample times, so the samples are made where they are consumed
(no host materialisation, no host-to-device copy), and the result stays on
the device, differentiable through magnus_gb300.autograd.
"""
from __future__ import annotations

from typing import Callable

import torch

from .autograd import magnus, magnus_sc


def sample_device(f: Callable, t0: float, tf: float, samples: int, *, dtype=torch.float32, device="cuda"):
    """f evaluated on the `samples` equally spaced times of [t0, tf] (a
    float64 CUDA tensor, as the reference's linspace), cast to `dtype`."""
    t = torch.linspace(float(t0), float(tf), int(samples), dtype=torch.float64, device=device)
    return torch.as_tensor(f(t), device=device).to(dtype).contiguous()


def compute_device(n: int, f: Callable, t0: float, tf: float, samples: int, *, op="sum", integrator="Auto",
                   precision="mixed", dtype=torch.float32, checkpoint_K=0, device="cuda"):
    """Magnus output of the matrix function f (torch-vectorized: a (S,)
    tensor of times -> (S, d, d)), sampled and computed on the GPU."""
    A = sample_device(f, t0, tf, samples, dtype=dtype, device=device)
    return magnus(A, n, t0, tf, op=op, integrator=integrator, precision=precision, checkpoint_K=checkpoint_K)


def compute_sc_device(n: int, f: Callable, t0: float, tf: float, samples: int, *, op="sum", integrator="Auto",
                      precision="mixed", dtype=torch.float32, checkpoint_K=0, device="cuda"):
    """SpaceCurve form of compute_device (f: times -> (S, 3))."""
    F = sample_device(f, t0, tf, samples, dtype=dtype, device=device)
    return magnus_sc(F, n, t0, tf, op=op, integrator=integrator, precision=precision, checkpoint_K=checkpoint_K)


def expm(omega):
    """Matrix exponential of Omega (..., d, d) on its device (the consumer of
    a Magnus sum: the propagator exp(Omega)); batched, differentiable."""
    return torch.linalg.matrix_exp(omega)
