"""Generates the golden fixtures in this directory from the reference
implementation itself (s-cavalier/magnus-dp compiled from its own sources by
oracle/build_ref.sh into oracle/_ref/).

Run from the repository root:   python tests/golden/make_golden.py

Every case stores its inputs and the reference's outputs, computed with the
serial Gauss-Legendre backend and the Fixed2 / Manual / SpaceCurve policies
(exact reference arithmetic; the Blas policy is MKL-dependent and not used).
The fixtures are read by tests/ only; nothing at run time needs the
reference.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, os.path.join(ROOT, "magnus-dp_gb300"))

import magnus  # noqa: E402  (the reference, from oracle/_ref)
from magnus_gb300 import workloads  # noqa: E402

core = magnus._core


def backend(d):
    return "Fixed2" if d == 2 else "Manual"


def small_cases():
    rng = np.random.default_rng(1234)
    cases = {}
    idx = 0
    for integ, S in [("Boole", 17), ("Simpson", 13), ("Trapezoid", 11), ("Riemann", 10)]:
        for d in (2, 3, 5):
            A = rng.standard_normal((S, d, d)) / np.sqrt(d)
            for n in (1, 2, 4, 6):
                for op in ("one", "many", "sum"):
                    key = f"m{idx:03d}"
                    idx += 1
                    out = core.compute(n, A, 0.0, 1.3, op=op, matrix_backend=backend(d), integrator=integ,
                                       gl_backend="serial")
                    cot = rng.standard_normal(out.shape)
                    dA = core.compute_vjp(n, A, cot, t0=0.0, tf=1.3, op=op, matrix_backend=backend(d),
                                          integrator=integ)
                    cases[key] = dict(kind="matrix", integrator=integ, op=op, n=n, t0=0.0, tf=1.3, A=A, out=out,
                                      cot=cot, dA=dA)
                    if n == 4 and op == "sum":
                        _, carry = core.compute(n, A, 0.0, 1.3, op=op, matrix_backend=backend(d), integrator=integ,
                                                gl_backend="serial", record_vjp=True)
                        cases[key]["carry"] = carry
        F = rng.standard_normal((S, 3))
        for n in (1, 2, 4, 6):
            for op in ("one", "many", "sum"):
                key = f"s{idx:03d}"
                idx += 1
                out = core.compute_sc(n, F, 0.0, 2.0, op=op, integrator=integ, gl_backend="serial")
                cot = rng.standard_normal(out.shape)
                dA = core.compute_sc_vjp(n, F, cot, t0=0.0, tf=2.0, op=op, integrator=integ)
                cases[key] = dict(kind="spacecurve", integrator=integ, op=op, n=n, t0=0.0, tf=2.0, A=F, out=out,
                                  cot=cot, dA=dA)
                if n == 4 and op == "many":
                    _, carry = core.compute_sc(n, F, 0.0, 2.0, op=op, integrator=integ, gl_backend="serial",
                                               record_vjp=True)
                    cases[key]["carry"] = carry
    return cases


def medium_cases():
    """Multi-chunk sizes (the engine's default chunk is 256 samples; tests
    also force small chunks)."""
    rng = np.random.default_rng(99)
    cases = {}
    for key, (integ, S, d, n, op) in {
        "md16": ("Boole", 261, 16, 5, "sum"),
        "md8s": ("Simpson", 301, 8, 4, "many"),
        "md4t": ("Trapezoid", 257, 4, 3, "one"),
        "md3r": ("Riemann", 300, 3, 6, "many"),
    }.items():
        A = rng.standard_normal((S, d, d)) / np.sqrt(d)
        out = core.compute(n, A, 0.0, 1.0, op=op, matrix_backend=backend(d), integrator=integ, gl_backend="serial")
        cot = rng.standard_normal(out.shape)
        dA = core.compute_vjp(n, A, cot, t0=0.0, tf=1.0, op=op, matrix_backend=backend(d), integrator=integ)
        cases[key] = dict(kind="matrix", integrator=integ, op=op, n=n, t0=0.0, tf=1.0, A=A, out=out, cot=cot, dA=dA)
    F = workloads.config1_samples_np(*workloads.config1_coeffs(seed=1, batch=1), samples=1025, dtype=np.float64)[0]
    out = core.compute_sc(6, F, 0.0, 2.0, op="many", integrator="Simpson", gl_backend="serial")
    cot = rng.standard_normal(out.shape)
    dA = core.compute_sc_vjp(6, F, cot, t0=0.0, tf=2.0, op="many", integrator="Simpson")
    cases["mdsc"] = dict(kind="spacecurve", integrator="Simpson", op="many", n=6, t0=0.0, tf=2.0, A=F, out=out,
                         cot=cot, dA=dA)
    return cases


def config0_cases():
    A = workloads.config0_samples(seed=0)
    cases = {}
    for op in ("sum", "many"):
        out = core.compute(4, A, 0.0, 1.0, op=op, matrix_backend="Fixed2", integrator="Boole", gl_backend="serial")
        cases[f"cfg0_{op}"] = dict(kind="matrix", integrator="Boole", op=op, n=4, t0=0.0, tf=1.0, A=A, out=out)
    return cases


def float32_cases():
    """Reference float32 runs next to the float64 run on the upcast input
    (the float64 run is the accuracy oracle for float32 data)."""
    rng = np.random.default_rng(7)
    A32 = (rng.standard_normal((129, 4, 4)) / 2).astype(np.float32)
    cases = {}
    out32 = core.compute(5, A32, 0.0, 1.0, op="many", matrix_backend="Manual", integrator="Boole", gl_backend="serial")
    out64 = core.compute(5, A32.astype(np.float64), 0.0, 1.0, op="many", matrix_backend="Manual", integrator="Boole",
                         gl_backend="serial")
    cases["f32"] = dict(kind="matrix", integrator="Boole", op="many", n=5, t0=0.0, tf=1.0, A=A32, out=out32,
                        out64=out64)
    return cases


def complex_cases():
    """Complex matrix problems (the reference's complex64 / complex128
    kernels): forward, bilinear VJP, one carry record, and a complex64 run
    next to the complex128 run on the upcast input."""
    rng = np.random.default_rng(11)
    cases = {}
    idx = 0
    for integ, S in [("Boole", 17), ("Simpson", 13), ("Trapezoid", 11), ("Riemann", 10)]:
        for d in (2, 3):
            A = (rng.standard_normal((S, d, d)) + 1j * rng.standard_normal((S, d, d))) / np.sqrt(2 * d)
            for n in (1, 3, 5):
                for op in ("one", "many", "sum"):
                    key = f"c{idx:03d}"
                    idx += 1
                    out = core.compute(n, A, 0.0, 1.3, op=op, matrix_backend=backend(d), integrator=integ,
                                       gl_backend="serial")
                    cot = rng.standard_normal(out.shape) + 1j * rng.standard_normal(out.shape)
                    dA = core.compute_vjp(n, A, cot, t0=0.0, tf=1.3, op=op, matrix_backend=backend(d),
                                          integrator=integ)
                    cases[key] = dict(kind="matrix", integrator=integ, op=op, n=n, t0=0.0, tf=1.3, A=A, out=out,
                                      cot=cot, dA=dA)
            _, carry = core.compute(4, A, 0.0, 1.3, op="sum", matrix_backend=backend(d), integrator=integ,
                                    gl_backend="serial", record_vjp=True)
            out = core.compute(4, A, 0.0, 1.3, op="sum", matrix_backend=backend(d), integrator=integ,
                               gl_backend="serial")
            cases[f"carry_{integ}_{d}"] = dict(kind="matrix", integrator=integ, op="sum", n=4, t0=0.0, tf=1.3, A=A,
                                               out=out, carry=carry)
    for integ, S in [("Boole", 17), ("Simpson", 13), ("Trapezoid", 11), ("Riemann", 10)]:
        F = (rng.standard_normal((S, 3)) + 1j * rng.standard_normal((S, 3))) / 2
        for n in (1, 2, 5):
            for op in ("one", "many", "sum"):
                key = f"z{idx:03d}"
                idx += 1
                out = core.compute_sc(n, F, 0.0, 1.3, op=op, integrator=integ, gl_backend="serial")
                cot = rng.standard_normal(out.shape) + 1j * rng.standard_normal(out.shape)
                dA = core.compute_sc_vjp(n, F, cot, t0=0.0, tf=1.3, op=op, integrator=integ)
                cases[key] = dict(kind="spacecurve", integrator=integ, op=op, n=n, t0=0.0, tf=1.3, A=F, out=out,
                                  cot=cot, dA=dA)
        out, carry = core.compute_sc(4, F, 0.0, 1.3, op="sum", integrator=integ, gl_backend="serial",
                                     record_vjp=True)
        cases[f"sccarry_{integ}"] = dict(kind="spacecurve", integrator=integ, op="sum", n=4, t0=0.0, tf=1.3, A=F,
                                         out=out, carry=carry)
    A64 = (rng.standard_normal((129, 4, 4)) + 1j * rng.standard_normal((129, 4, 4))) / 3
    A32 = A64.astype(np.complex64)
    out32 = core.compute(5, A32, 0.0, 1.0, op="many", matrix_backend="Manual", integrator="Boole", gl_backend="serial")
    out64 = core.compute(5, A32.astype(np.complex128), 0.0, 1.0, op="many", matrix_backend="Manual",
                         integrator="Boole", gl_backend="serial")
    cases["c64"] = dict(kind="matrix", integrator="Boole", op="many", n=5, t0=0.0, tf=1.0, A=A32, out=out32,
                        out64=out64)
    return cases


def config4_full_cases():
    """One full trajectory of config4's shape (d = 32, S = 32769, n = 5,
    Boole) run by the reference in FP64: every order (op many) and dA of op
    sum at 39 sample indices (the ends, chunk boundaries of the engine's
    256-sample checkpoints, and evenly spaced ones).  The samples are a cubic
    polynomial in t with seeded coefficients, rounded to float32, so that the
    tests regenerate them bit for bit on any machine (only +, *, and the
    float32 cast; the benchmark's cos term would depend on the platform's
    libm); the 268 MB of samples are not stored."""
    d, S, n = 32, 32769, 5
    A64 = workloads.config4_poly_samples(seed=44, samples=S, d=d)
    out = core.compute(n, A64, 0.0, 1.0, op="many", matrix_backend="Manual", integrator="Boole", gl_backend="serial")
    cot = workloads.config4_cotangent(batch=1, d=d)[0].astype(np.float64)
    dA = core.compute_vjp(n, A64, cot, t0=0.0, tf=1.0, op="sum", matrix_backend="Manual", integrator="Boole")
    idx = sorted(set([0, 1, 2, 3, 4, 255, 256, 257, 258, 511, 512, 513, 16384, 16385, S - 2, S - 1]
                     + [int(v) for v in np.linspace(0, S - 1, 25)]))
    return {"c4full": dict(kind="matrix", integrator="Boole", op="many", n=n, t0=0.0, tf=1.0, seed=44, samples=S,
                           dim=d, out=out, cot=cot, idx=np.array(idx), dA_rows=dA[idx],
                           dA_norm=np.linalg.norm(dA))}


def config2_full_cases():
    """One full trajectory of config2's shape (skew-symmetric d = 64, S =
    16385, n = 4, Boole) run by the reference in FP64, stored like
    config4_full_cases (every order, dA at sample indices; samples a seeded
    skew quadratic in t, regenerated bit for bit by the tests)."""
    d, S, n = 64, 16385, 4
    A64 = workloads.config2_poly_samples(seed=22, samples=S, d=d)
    out = core.compute(n, A64, 0.0, 1.0, op="many", matrix_backend="Manual", integrator="Boole", gl_backend="serial")
    cot = np.random.default_rng(23).standard_normal((d, d))
    dA = core.compute_vjp(n, A64, cot, t0=0.0, tf=1.0, op="sum", matrix_backend="Manual", integrator="Boole")
    idx = sorted(set([0, 1, 2, 3, 4, 255, 256, 257, 258, 8192, 8193, S - 2, S - 1]
                     + [int(v) for v in np.linspace(0, S - 1, 17)]))
    return {"c2full": dict(kind="matrix", integrator="Boole", op="many", n=n, t0=0.0, tf=1.0, seed=22, samples=S,
                           dim=d, out=out, cot=cot, idx=np.array(idx), dA_rows=dA[idx],
                           dA_norm=np.linalg.norm(dA))}


def save(name, cases):
    flat = {}
    for key, c in cases.items():
        for field, value in c.items():
            flat[f"{key}/{field}"] = np.asarray(value)
    np.savez_compressed(os.path.join(HERE, name), **flat)


def main():
    makers = {"small.npz": small_cases, "medium.npz": medium_cases, "config0.npz": config0_cases,
              "float32.npz": float32_cases, "complex.npz": complex_cases, "config4_full.npz": config4_full_cases,
              "config2_full.npz": config2_full_cases}
    for name in (sys.argv[1:] or makers):  # e.g. `make_golden.py complex.npz` regenerates one file
        save(name, makers[name]())
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
