"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (no datasets are involved).

All random draws come from ``numpy.random.default_rng(seed)`` so they are the
same on every machine; the sampled matrices are evaluated from those draws
(numpy on the host, or torch on the GPU for the large batches).

  config0  d=2 float64, A(t) = C0 + C1 sin(w1 t) + C2 cos(w2 t), C_k ~ N(0, 1/d),
           w ~ U[0.5, 3]; t in [0, 1], S = 4097, Boole, n = 4.
  config1  SpaceCurve batch: f(t) = sum_{m=1..8} a_m sin(2 pi m t) + b_m cos(2 pi m t),
           a_m, b_m ~ N(0, 1/m^2) in R^3; t in [0, 2], S = 65537, Simpson, n = 6, many.
  config2  batch of d=64 A(t) = S0 + t S1 + sin(3t) S2, S_k skew-symmetric with upper
           entries ~ N(0, 1/d); t in [0, 1], S = 16385, Boole, n = 4, sum.
  config3  uneven batch: d in {2..128}, S = 4k+1 log-uniform in [257, 65537],
           n in 2..6, A as config0 at each d.
  config4  batch of d=32 A(t) = C0 + C1 t + C2 t^2 + C3 cos(5t), C_k ~ N(0, 1/d);
           S = 32769, Boole, n = 5, sum; cotangent ~ N(0, 1).
"""
from __future__ import annotations

import numpy as np


# ---------------------------------------------------------------- config0
def config0_coeffs(seed=0, d=2):
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((3, d, d)) * np.sqrt(1.0 / d)
    w = rng.uniform(0.5, 3.0, size=2)
    return C, w


def config0_samples(seed=0, d=2, samples=4097, t0=0.0, tf=1.0, dtype=np.float64):
    C, w = config0_coeffs(seed, d)
    t = np.linspace(t0, tf, samples)[:, None, None]
    A = C[0] + C[1] * np.sin(w[0] * t) + C[2] * np.cos(w[1] * t)
    return np.ascontiguousarray(A, dtype=dtype)


# ---------------------------------------------------------------- config1
def config1_coeffs(seed=1, batch=4096):
    rng = np.random.default_rng(seed)
    m = np.arange(1, 9, dtype=np.float64)
    a = rng.standard_normal((batch, 8, 3)) / m[None, :, None]
    b = rng.standard_normal((batch, 8, 3)) / m[None, :, None]
    return a, b


def config1_samples_np(a, b, samples=65537, t0=0.0, tf=2.0, dtype=np.float32):
    t = np.linspace(t0, tf, samples)
    m = np.arange(1, 9, dtype=np.float64)
    ang = 2 * np.pi * m[None, :] * t[:, None]  # (S, 8)
    F = np.einsum("sm,bmc->bsc", np.sin(ang), a) + np.einsum("sm,bmc->bsc", np.cos(ang), b)
    return np.ascontiguousarray(F, dtype=dtype)


def config1_samples_torch(a, b, samples=65537, t0=0.0, tf=2.0, dtype=None, device="cuda"):
    import torch
    dtype = dtype or torch.float32
    t = torch.linspace(t0, tf, samples, dtype=torch.float64, device=device)
    m = torch.arange(1, 9, dtype=torch.float64, device=device)
    ang = 2 * np.pi * m[None, :] * t[:, None]
    ta = torch.as_tensor(a, device=device)
    tb = torch.as_tensor(b, device=device)
    out = torch.empty((a.shape[0], samples, 3), dtype=dtype, device=device)
    step = 256
    for i in range(0, a.shape[0], step):
        F = torch.einsum("sm,bmc->bsc", torch.sin(ang), ta[i:i + step]) + \
            torch.einsum("sm,bmc->bsc", torch.cos(ang), tb[i:i + step])
        out[i:i + step] = F.to(dtype)
    return out


# ---------------------------------------------------------------- config2
def config2_coeffs(seed=2, batch=256, d=64):
    rng = np.random.default_rng(seed)
    U = rng.standard_normal((batch, 3, d, d)) * np.sqrt(1.0 / d)
    Sk = np.triu(U, 1)
    return Sk - np.swapaxes(Sk, -1, -2)


def config2_samples_torch(Sk, samples=16385, t0=0.0, tf=1.0, dtype=None, device="cuda"):
    import torch
    dtype = dtype or torch.float32
    t = torch.linspace(t0, tf, samples, dtype=torch.float64, device=device)
    basis = torch.stack([torch.ones_like(t), t, torch.sin(3 * t)], dim=1)  # (S, 3)
    S3 = torch.as_tensor(Sk, device=device)
    out = torch.empty((Sk.shape[0], samples, Sk.shape[-1], Sk.shape[-1]), dtype=dtype, device=device)
    for i in range(Sk.shape[0]):
        out[i] = torch.einsum("sk,kij->sij", basis, S3[i]).to(dtype)
    return out


def config2_poly_samples(seed=22, samples=16385, d=64, t0=0.0, tf=1.0):
    """One trajectory of config2's shape with the skew-symmetric A(t) = S0 +
    t (S1 + t S2) (config2's seeded skew coefficients): elementwise float64
    + and * only, so bit-identical on every platform (and exactly skew),
    rounded to float32 and returned as float64."""
    Sk = config2_coeffs(seed=seed, batch=1, d=d)[0]
    t = np.linspace(t0, tf, samples)[:, None, None]
    A = Sk[0] + t * (Sk[1] + t * Sk[2])
    return A.astype(np.float32).astype(np.float64)


# ---------------------------------------------------------------- config4
def config4_coeffs(seed=4, batch=512, d=32):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((batch, 4, d, d)) * np.sqrt(1.0 / d)


def config4_basis_np(samples=32769, t0=0.0, tf=1.0):
    t = np.linspace(t0, tf, samples)
    return np.stack([np.ones_like(t), t, t * t, np.cos(5 * t)], axis=1)


def config4_samples_np(Ck, samples=32769, t0=0.0, tf=1.0, dtype=np.float32):
    basis = config4_basis_np(samples, t0, tf)
    return np.ascontiguousarray(np.einsum("sk,bkij->bsij", basis, Ck), dtype=dtype)


def config4_samples_torch(Ck, samples=32769, t0=0.0, tf=1.0, dtype=None, device="cuda", out=None):
    import torch
    dtype = dtype or torch.float32
    t = torch.linspace(t0, tf, samples, dtype=torch.float64, device=device)
    basis = torch.stack([torch.ones_like(t), t, t * t, torch.cos(5 * t)], dim=1)
    C = torch.as_tensor(Ck, device=device)
    if out is None:
        out = torch.empty((Ck.shape[0], samples, Ck.shape[-1], Ck.shape[-1]), dtype=dtype, device=device)
    for i in range(Ck.shape[0]):
        out[i] = torch.einsum("sk,kij->sij", basis, C[i]).to(dtype)
    return out


def config4_poly_samples(seed=44, samples=32769, d=32, t0=0.0, tf=1.0):
    """One trajectory of config4's shape with A(t) = C0 + t (C1 + t (C2 + t
    C3)), C_k ~ N(0, 1/d) seeded: evaluated with elementwise float64 + and *
    only, so bit-identical on every platform, then rounded to float32 and
    returned as float64 (the exact float32 values)."""
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((4, d, d)) * np.sqrt(1.0 / d)
    t = np.linspace(t0, tf, samples)[:, None, None]
    A = C[0] + t * (C[1] + t * (C[2] + t * C[3]))
    return A.astype(np.float32).astype(np.float64)


def config4_cotangent(seed=40, batch=512, d=32, dtype=np.float32):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((batch, d, d)).astype(dtype)


# ---------------------------------------------------------------- config3
def config3_instances(seed=3, count=10000):
    """Per-instance (d, S, n) of the uneven batch and its config0-style
    coefficient seeds."""
    rng = np.random.default_rng(seed)
    ds = rng.choice(np.array([2, 4, 8, 16, 32, 64, 128]), size=count)
    lo, hi = np.log(257.0), np.log(65537.0)
    S = np.exp(rng.uniform(lo, hi, size=count))
    S = (np.round((S - 1) / 4) * 4 + 1).astype(np.int64)
    S = np.clip(S, 257, 65537)
    ns = rng.integers(2, 7, size=count)
    seeds = rng.integers(0, 2**31 - 1, size=count)
    return ds, S, ns, seeds
