"""Parity at the benchmarked configuration sizes, per order.

One full-size instance of each configuration goes through the engine's
public array entry points (host arrays -> C ABI) and is compared with the
collapsed FP64 checker (oracle/collapsed.py, pinned against the C oracle by
tests/test_collapsed_cpu.py) or, for 2 x 2 and SpaceCurve data, the C oracle
itself.  The long sample axes here (16385 .. 65537 samples, 64 .. 256 chunk
steps) are where rounding in the prefix scans and the chunk carries would
grow, so every order is checked separately.

Tolerances (relative Frobenius, per order):
  plain form, float64 input       <= 1e-12  (against the FP64 checker)
  mixed form, float32 input       <= 1e-6   (against the checker on the upcast input)
Orders that vanish analytically (below 1e-6 of the largest order) are
measured against the largest order's norm.
"""
import numpy as np
import pytest

import collapsed as Cl
import magnus_gb300 as magnus
import oracle as O
from magnus_gb300 import workloads

pytestmark = pytest.mark.gpu
core = magnus._core
PLAIN_TOL = 1e-12
MIXED_TOL = 1e-6


def order_errors(out, ref):
    out = np.asarray(out, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = max(np.linalg.norm(r) for r in ref)
    errs = []
    for k in range(ref.shape[0]):
        nk = np.linalg.norm(ref[k])
        errs.append(float(np.linalg.norm(out[k] - ref[k]) / (nk if nk >= 1e-6 * scale else scale)))
    return errs


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def check_matrix(A32, n, integrator, tf, cot, K=0):
    """Plain (float64 in) and mixed (float32 in) forward per order and VJP
    (op sum) against the collapsed checker on the float64 upcast."""
    A64 = A32.astype(np.float64)
    ref = Cl.forward(A64, n, 0.0, tf, "many", integrator)
    gref = Cl.vjp(A64, cot.astype(np.float64), n, 0.0, tf, "sum", integrator)
    out_p = core.compute(n, A64, 0.0, tf, op="many", integrator=integrator, precision="plain", checkpoint_K=K)
    g_p = core.compute_vjp(n, A64, cot.astype(np.float64), t0=0.0, tf=tf, op="sum", integrator=integrator,
                           precision="plain", checkpoint_K=K)
    out_m = core.compute(n, A32, 0.0, tf, op="many", integrator=integrator, precision="mixed", checkpoint_K=K)
    g_m = core.compute_vjp(n, A32, cot.astype(np.float32), t0=0.0, tf=tf, op="sum", integrator=integrator,
                           precision="mixed", checkpoint_K=K)
    ep, em = order_errors(out_p, ref), order_errors(out_m, ref)
    gp, gm = rel(g_p, gref), rel(g_m, gref)
    print(f"plain per order {ep} dA {gp:.2e}; mixed per order {em} dA {gm:.2e}")
    assert max(ep) <= PLAIN_TOL, ep
    assert gp <= PLAIN_TOL, gp
    assert max(em) <= MIXED_TOL, em
    assert gm <= MIXED_TOL, gm


def test_config4_full_instance(cuda):
    """Config4: d = 32, S = 32769, Boole, n = 5 (128 chunk steps at the
    default checkpoint interval), the bench's first trajectory and
    cotangent."""
    Ck = workloads.config4_coeffs(seed=4, batch=1, d=32)
    A32 = workloads.config4_samples_np(Ck, samples=32769, dtype=np.float32)[0]
    cot = workloads.config4_cotangent(batch=1, d=32)[0]
    check_matrix(A32, 5, "Boole", 1.0, cot)


def config2_instance(seed=2, d=64, samples=16385):
    Sk = workloads.config2_coeffs(seed=seed, batch=1, d=d)[0]
    t = np.linspace(0.0, 1.0, samples)[:, None, None]
    return np.ascontiguousarray(Sk[0] + t * Sk[1] + np.sin(3 * t) * Sk[2], dtype=np.float32)


def test_config2_full_instance(cuda):
    """Config2: skew-symmetric d = 64, S = 16385, Boole, n = 4 (the
    tensor-core kernel in the mixed form)."""
    A32 = config2_instance()
    cot = np.random.default_rng(22).standard_normal((64, 64))
    check_matrix(A32, 4, "Boole", 1.0, cot)


@pytest.mark.parametrize("d,S,n", [(128, 8193, 6), (64, 16385, 6), (16, 65537, 6), (32, 65537, 3)])
def test_config3_extreme_shapes(d, S, n, cuda):
    """Config3's extremes: the largest dimension at the longest sample count
    the FP64 checker affords, and the longest sample count at smaller d,
    A(t) as config0 at each d, float32 in."""
    A32 = workloads.config0_samples(seed=300 + d, d=d, samples=S).astype(np.float32)
    cot = np.random.default_rng(d).standard_normal((d, d))
    check_matrix(A32, n, "Boole", 1.0, cot)


def test_config3_two_by_two_longest(cuda):
    """2 x 2 matrices at S = 65537, n = 6 against the C oracle (per-node
    recursion) in both forms."""
    A64 = workloads.config0_samples(seed=302, d=2, samples=65537)
    A32 = A64.astype(np.float32)
    ref = O.forward(A32.astype(np.float64), 6, 0.0, 1.0, "many", "Boole")
    out_p = core.compute(6, A32.astype(np.float64), 0.0, 1.0, op="many", integrator="Boole", precision="plain")
    out_m = core.compute(6, A32, 0.0, 1.0, op="many", integrator="Boole", precision="mixed")
    assert max(order_errors(out_p, ref)) <= PLAIN_TOL
    assert max(order_errors(out_m, ref)) <= MIXED_TOL
    cot = np.random.default_rng(2).standard_normal((2, 2))
    gref = O.vjp(A32.astype(np.float64), cot, 6, 0.0, 1.0, "sum", "Boole")
    assert rel(core.compute_vjp(6, A32.astype(np.float64), cot, op="sum", integrator="Boole"), gref) <= PLAIN_TOL
    assert rel(core.compute_vjp(6, A32, cot.astype(np.float32), op="sum", integrator="Boole", precision="mixed"),
               gref) <= MIXED_TOL


def test_config1_full_spacecurve(cuda):
    """Config1: one SpaceCurve, S = 65537 on [0, 2], Simpson, n = 6, op many,
    against the C oracle in both forms (Omega_1 of whole-period sinusoids
    vanishes and is measured against the largest order)."""
    a, b = workloads.config1_coeffs(seed=1, batch=1)
    F32 = workloads.config1_samples_np(a, b, samples=65537, dtype=np.float32)[0]
    F64 = F32.astype(np.float64)
    ref = O.forward_sc(F64, 6, 0.0, 2.0, "many", "Simpson")
    out_p = core.compute_sc(6, F64, 0.0, 2.0, op="many", integrator="Simpson", precision="plain")
    out_m = core.compute_sc(6, F32, 0.0, 2.0, op="many", integrator="Simpson", precision="mixed")
    ep, em = order_errors(out_p, ref), order_errors(out_m, ref)
    print(f"plain per order {ep}; mixed per order {em}")
    assert max(ep) <= PLAIN_TOL, ep
    assert max(em) <= MIXED_TOL, em
    cot = np.random.default_rng(1).standard_normal((6, 3))
    gref = O.vjp_sc(F64, cot, 6, 0.0, 2.0, "many", "Simpson")
    assert rel(core.compute_sc_vjp(6, F64, cot, t0=0.0, tf=2.0, op="many", integrator="Simpson"), gref) <= PLAIN_TOL
    assert rel(core.compute_sc_vjp(6, F32, cot.astype(np.float32), t0=0.0, tf=2.0, op="many", integrator="Simpson",
                                   precision="mixed"), gref) <= MIXED_TOL


def test_config4_size_against_reference_outputs(cuda):
    """The engine against the reference's own outputs at config4's size
    (tests/golden/config4_full.npz, written by the reference's module: every
    order and dA at 39 sample indices of one d = 32, S = 32769, n = 5 Boole
    trajectory whose samples are regenerated bit for bit here)."""
    from conftest import load_cases
    g = load_cases("config4_full.npz")["c4full"]
    n, S, d = int(g["n"]), int(g["samples"]), int(g["dim"])
    A64 = workloads.config4_poly_samples(seed=int(g["seed"]), samples=S, d=d)
    A32 = A64.astype(np.float32)
    idx = g["idx"]
    out_p = core.compute(n, A64, 0.0, 1.0, op="many", integrator="Boole", precision="plain")
    g_p = core.compute_vjp(n, A64, g["cot"], t0=0.0, tf=1.0, op="sum", integrator="Boole", precision="plain")
    out_m = core.compute(n, A32, 0.0, 1.0, op="many", integrator="Boole", precision="mixed")
    g_m = core.compute_vjp(n, A32, g["cot"].astype(np.float32), t0=0.0, tf=1.0, op="sum", integrator="Boole",
                           precision="mixed")
    ep, em = order_errors(out_p, g["out"]), order_errors(out_m, g["out"])
    gp, gm = rel(g_p[idx], g["dA_rows"]), rel(g_m[idx], g["dA_rows"])
    print(f"vs reference: plain per order {ep} dA {gp:.2e}; mixed per order {em} dA {gm:.2e}")
    assert max(ep) <= PLAIN_TOL and gp <= PLAIN_TOL, (ep, gp)
    assert max(em) <= MIXED_TOL and gm <= MIXED_TOL, (em, gm)


def test_config2_size_against_reference_outputs(cuda):
    """The engine against the reference's own outputs at config2's size
    (tests/golden/config2_full.npz: one skew-symmetric d = 64, S = 16385,
    n = 4 Boole trajectory, samples regenerated bit for bit here)."""
    from conftest import load_cases
    g = load_cases("config2_full.npz")["c2full"]
    n, S, d = int(g["n"]), int(g["samples"]), int(g["dim"])
    A64 = workloads.config2_poly_samples(seed=int(g["seed"]), samples=S, d=d)
    A32 = A64.astype(np.float32)
    idx = g["idx"]
    out_p = core.compute(n, A64, 0.0, 1.0, op="many", integrator="Boole", precision="plain")
    g_p = core.compute_vjp(n, A64, g["cot"], t0=0.0, tf=1.0, op="sum", integrator="Boole", precision="plain")
    out_m = core.compute(n, A32, 0.0, 1.0, op="many", integrator="Boole", precision="mixed")
    g_m = core.compute_vjp(n, A32, g["cot"].astype(np.float32), t0=0.0, tf=1.0, op="sum", integrator="Boole",
                           precision="mixed")
    ep, em = order_errors(out_p, g["out"]), order_errors(out_m, g["out"])
    gp, gm = rel(g_p[idx], g["dA_rows"]), rel(g_m[idx], g["dA_rows"])
    print(f"vs reference: plain per order {ep} dA {gp:.2e}; mixed per order {em} dA {gm:.2e}")
    assert max(ep) <= PLAIN_TOL and gp <= PLAIN_TOL, (ep, gp)
    assert max(em) <= MIXED_TOL and gm <= MIXED_TOL, (em, gm)
