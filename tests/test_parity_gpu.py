"""GPU parity of the GB300 engine against the reference (golden fixtures made
by the reference itself) and the CPU oracle.

Tolerances (relative Frobenius):
  plain FP64 path   <= 1e-12 against the reference (the parity bar)
  mixed path        <= 1e-6  against the FP64 oracle (FP32 products, FP64 carries)
  float32 inputs    <= 2e-6  against the FP64 oracle on the upcast input
"""
import numpy as np
import pytest

import magnus_gb300 as magnus
import oracle as O
from conftest import load_cases, rel

pytestmark = pytest.mark.gpu

SMALL = load_cases("small.npz")
MEDIUM = load_cases("medium.npz")
PLAIN_TOL = 1e-12
core = magnus._core


def run_fwd(c, K=0, precision="plain", record=False):
    if c["kind"] == "matrix":
        return core.compute(c["n"], c["A"], c["t0"], c["tf"], op=c["op"], integrator=c["integrator"],
                            record_vjp=record, precision=precision, checkpoint_K=K)
    return core.compute_sc(c["n"], c["A"], c["t0"], c["tf"], op=c["op"], integrator=c["integrator"],
                           record_vjp=record, precision=precision, checkpoint_K=K)


def run_vjp(c, K=0, precision="plain"):
    if c["kind"] == "matrix":
        return core.compute_vjp(c["n"], c["A"], c["cot"], t0=c["t0"], tf=c["tf"], op=c["op"],
                                integrator=c["integrator"], precision=precision, checkpoint_K=K)
    return core.compute_sc_vjp(c["n"], c["A"], c["cot"], t0=c["t0"], tf=c["tf"], op=c["op"],
                               integrator=c["integrator"], precision=precision, checkpoint_K=K)


@pytest.mark.parametrize("K", [0, 4, 8])
@pytest.mark.parametrize("key", sorted(SMALL))
def test_small_cases_match_reference(key, K, cuda):
    c = SMALL[key]
    out = run_fwd(c, K)
    assert out.shape == c["out"].shape
    assert rel(out, c["out"]) <= PLAIN_TOL, (key, rel(out, c["out"]))
    dA = run_vjp(c, K)
    assert dA.shape == c["dA"].shape
    assert rel(dA, c["dA"]) <= PLAIN_TOL, (key, rel(dA, c["dA"]))


@pytest.mark.parametrize("K", [0, 4, 32])
@pytest.mark.parametrize("key", sorted(k for k, c in SMALL.items() if "carry" in c))
def test_carry_matches_reference(key, K, cuda):
    c = SMALL[key]
    out, carry = run_fwd(c, K, record=True)
    assert carry.shape == c["carry"].shape
    assert rel(out, c["out"]) <= PLAIN_TOL
    assert rel(carry, c["carry"]) <= PLAIN_TOL, rel(carry, c["carry"])


@pytest.mark.parametrize("K", [0, 12, 64])
@pytest.mark.parametrize("key", sorted(MEDIUM))
def test_medium_cases_match_reference(key, K, cuda):
    c = MEDIUM[key]
    assert rel(run_fwd(c, K), c["out"]) <= PLAIN_TOL
    assert rel(run_vjp(c, K), c["dA"]) <= PLAIN_TOL


def test_config0_matches_reference(cuda):
    for c in load_cases("config0.npz").values():
        out = run_fwd(c)
        assert rel(out, c["out"]) <= PLAIN_TOL, rel(out, c["out"])


def test_float32_input_against_fp64_oracle(cuda):
    c = load_cases("float32.npz")["f32"]
    out = run_fwd(c)
    assert out.dtype == np.float32
    assert rel(out, c["out64"]) <= 2e-6
    out_mixed = run_fwd(c, precision="mixed")
    assert rel(out_mixed, c["out64"]) <= 2e-6


def smooth_samples(S, d, seed):
    """config0-style smooth A(t) at dimension d (the benchmark inputs' form)."""
    from magnus_gb300 import workloads
    return workloads.config0_samples(seed=seed, d=d, samples=S)


@pytest.mark.parametrize("integrator,S", [("Boole", 1025), ("Simpson", 1025), ("Trapezoid", 1023), ("Riemann", 1000)])
@pytest.mark.parametrize("d", [2, 8, 32])
def test_mixed_precision_within_1e6_per_order(integrator, S, d, cuda):
    """Mixed form (FP32 products, FP64 carries) on smooth inputs: every order
    within 1e-6 of the FP64 oracle, and the VJP too."""
    rng = np.random.default_rng(d * 7 + S)
    A = smooth_samples(S, d, seed=d)
    n = 5
    ref = O.forward(A, n, 0.0, 1.0, "many", integrator)
    out = core.compute(n, A, 0.0, 1.0, op="many", integrator=integrator, precision="mixed")
    for k in range(n):
        assert rel(out[k], ref[k]) <= 1e-6, (k, rel(out[k], ref[k]))
    cot = rng.standard_normal((d, d))
    gref = O.vjp(A, cot, n, 0.0, 1.0, "sum", integrator)
    g = core.compute_vjp(n, A, cot, t0=0.0, tf=1.0, op="sum", integrator=integrator, precision="mixed")
    assert rel(g, gref) <= 1e-6, rel(g, gref)


@pytest.mark.parametrize("d", [2, 8, 32])
def test_mixed_precision_rough_input_normwise(d, cuda):
    """White-noise samples make the high orders nearly cancel; normwise over
    all orders the mixed form still stays within 1e-6."""
    rng = np.random.default_rng(d)
    A = rng.standard_normal((1025, d, d)) / np.sqrt(d)
    ref = O.forward(A, 5, 0.0, 1.0, "many", "Boole")
    out = core.compute(5, A, 0.0, 1.0, op="many", integrator="Boole", precision="mixed")
    assert rel(out, ref) <= 1e-6


def test_mixed_spacecurve_within_1e6(cuda):
    from magnus_gb300 import workloads
    F = workloads.config1_samples_np(*workloads.config1_coeffs(seed=11, batch=1), samples=4097,
                                     dtype=np.float64)[0]
    ref = O.forward_sc(F, 6, 0.0, 2.0, "many", "Simpson")
    out = core.compute_sc(6, F, 0.0, 2.0, op="many", integrator="Simpson", precision="mixed")
    scale = max(np.linalg.norm(r) for r in ref)
    for k in range(6):
        # Omega_1 of whole-period sinusoids is zero analytically (~1e-15 here):
        # orders that vanish are measured against the largest order instead.
        den = np.linalg.norm(ref[k]) if np.linalg.norm(ref[k]) >= 1e-6 * scale else scale
        err = np.linalg.norm(out[k] - ref[k]) / den
        assert err <= 1e-6, (k, err)


@pytest.mark.parametrize("op", ["one", "many", "sum"])
@pytest.mark.parametrize("integrator", ["Riemann", "Trapezoid", "Simpson", "Boole"])
def test_vjp_matches_central_finite_difference(op, integrator, cuda):
    """Directional FD check in FP64, as the reference's own tests do
    (tests/test_python_api.py:64-147)."""
    samples = 17 if integrator != "Riemann" else 16
    rng = np.random.default_rng(3)
    data = rng.standard_normal((samples, 3, 3)) / 2
    direction = np.linspace(-0.3, 0.7, data.size).reshape(data.shape)
    n = 4
    out = core.compute(n, data, 0.0, 1.0, op=op, integrator=integrator)
    cot = np.linspace(0.2, 1.1, out.size).reshape(out.shape)
    g = core.compute_vjp(n, data, cot, t0=0.0, tf=1.0, op=op, integrator=integrator, checkpoint_K=4)
    eps = 1e-6
    plus = core.compute(n, data + eps * direction, 0.0, 1.0, op=op, integrator=integrator)
    minus = core.compute(n, data - eps * direction, 0.0, 1.0, op=op, integrator=integrator)
    expected = np.sum((plus - minus) * cot) / (2 * eps)
    np.testing.assert_allclose(np.sum(g * direction), expected, rtol=1e-7, atol=1e-9)


def test_vjp_with_reference_carry_equals_recompute(cuda):
    rng = np.random.default_rng(8)
    A = rng.standard_normal((33, 2, 2))
    f = lambda t: A  # noqa: E731
    out, carry = magnus.compute(4, f, 0.0, 1.0, 33, op="many", record_vjp=True)
    assert carry.shape == (3, 3, 33, 2, 2)
    cot = rng.standard_normal(out.shape)
    a = magnus.compute_vjp(4, f, cot, 0.0, 1.0, 33, op="many", vjp_data=carry)
    b = magnus.compute_vjp(4, f, cot, 0.0, 1.0, 33, op="many")
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12)
    ref_carry = O.forward(A, 4, 0.0, 1.0, "many", "Boole", record_vjp=True)[1]
    assert rel(carry, ref_carry) <= PLAIN_TOL


@pytest.mark.parametrize("integrator,S", [("Riemann", 2), ("Riemann", 3), ("Trapezoid", 3), ("Simpson", 3),
                                          ("Boole", 5)])
@pytest.mark.parametrize("n", [1, 2, 3])
def test_tiny_sample_counts(integrator, S, n, cuda):
    rng = np.random.default_rng(S * 10 + n)
    A = rng.standard_normal((S, 2, 2))
    ref = O.forward(A, n, 0.0, 1.0, "many", integrator)
    out = core.compute(n, A, 0.0, 1.0, op="many", integrator=integrator)
    assert rel(out, ref) <= PLAIN_TOL
    cot = rng.standard_normal(out.shape)
    assert rel(core.compute_vjp(n, A, cot, op="many", integrator=integrator),
               O.vjp(A, cot, n, 0.0, 1.0, "many", integrator)) <= PLAIN_TOL


@pytest.mark.parametrize("d", [1, 6, 7, 12, 40])
def test_uncommon_dimensions(d, cuda):
    rng = np.random.default_rng(d)
    A = rng.standard_normal((41, d, d)) / np.sqrt(d)
    ref = O.forward(A, 3, 0.0, 1.0, "many", "Boole")
    out = core.compute(3, A, 0.0, 1.0, op="many", integrator="Boole", checkpoint_K=8)
    assert rel(out, ref) <= PLAIN_TOL
    cot = rng.standard_normal((d, d))
    assert rel(core.compute_vjp(3, A, cot, integrator="Boole", checkpoint_K=8),
               O.vjp(A, cot, 3, 0.0, 1.0, "sum", "Boole")) <= PLAIN_TOL


def test_order_needing_a_larger_gl_table(cuda):
    rng = np.random.default_rng(2)
    A = rng.standard_normal((9, 2, 2)) / 4
    with pytest.raises(ValueError, match="exceeds GL table"):
        core.compute(130, A, 0.0, 1.0, integrator="Boole")
    magnus.replace_gl_table(70)
    try:
        out = core.compute(130, A, 0.0, 1.0, op="one", integrator="Boole")
        assert np.all(np.isfinite(out))
    finally:
        magnus.replace_gl_table(64)


@pytest.mark.parametrize("integrator,S", [("Boole", 1025), ("Simpson", 1023), ("Trapezoid", 1023), ("Riemann", 1000)])
@pytest.mark.parametrize("d", [16, 32])
@pytest.mark.parametrize("K", [0, 32])
def test_tiled_mixed_kernel_float32(integrator, S, d, K, cuda):
    """float32 inputs at d = 16 / 32 in mixed precision run the shared-memory
    tiled kernel; every order and the VJP stay within 1e-6 of FP64."""
    A = smooth_samples(S, d, seed=d + 1).astype(np.float32)
    A64 = A.astype(np.float64)
    n = 5
    ref = O.forward(A64, n, 0.0, 1.0, "many", integrator)
    out = core.compute(n, A, 0.0, 1.0, op="many", integrator=integrator, precision="mixed", checkpoint_K=K)
    assert out.dtype == np.float32
    for k in range(n):
        assert rel(out[k], ref[k]) <= 1e-6, (k, rel(out[k], ref[k]))
    rng = np.random.default_rng(d)
    cot = rng.standard_normal((d, d)).astype(np.float32)
    gref = O.vjp(A64, cot.astype(np.float64), n, 0.0, 1.0, "sum", integrator)
    g = core.compute_vjp(n, A, cot, t0=0.0, tf=1.0, op="sum", integrator=integrator, precision="mixed",
                         checkpoint_K=K)
    assert rel(g, gref) <= 1e-6, rel(g, gref)


@pytest.mark.parametrize("n", [1, 2, 3, 7])
def test_tiled_kernel_orders(n, cuda):
    A = smooth_samples(129, 32, seed=n).astype(np.float32)
    ref = O.forward(A.astype(np.float64), n, 0.0, 1.0, "many", "Boole")
    out = core.compute(n, A, 0.0, 1.0, op="many", integrator="Boole", precision="mixed", checkpoint_K=16)
    assert rel(out, ref) <= 1e-6
    cot = np.ones((32, 32), dtype=np.float32)
    gref = O.vjp(A.astype(np.float64), cot.astype(np.float64), n, 0.0, 1.0, "sum", "Boole")
    g = core.compute_vjp(n, A, cot, integrator="Boole", precision="mixed", checkpoint_K=16)
    assert rel(g, gref) <= 1e-6, rel(g, gref)


@pytest.mark.parametrize("integrator,S", [("Boole", 129), ("Simpson", 131), ("Trapezoid", 97), ("Riemann", 90)])
@pytest.mark.parametrize("d", [64, 128])
def test_big_mixed_kernel_float32(integrator, S, d, cuda):
    """float32 inputs at d = 64 / 128 in mixed precision run the tensor-core
    chunk kernel (mgb_bigtc.cu, tcgen05 on BF16 operand pieces); orders and
    VJP within 1e-6."""
    A = smooth_samples(S, d, seed=d + 5).astype(np.float32)
    A64 = A.astype(np.float64)
    n = 4
    ref = O.forward(A64, n, 0.0, 1.0, "many", integrator)
    out = core.compute(n, A, 0.0, 1.0, op="many", integrator=integrator, precision="mixed", checkpoint_K=32)
    for k in range(n):
        assert rel(out[k], ref[k]) <= 1e-6, (k, rel(out[k], ref[k]))
    rng = np.random.default_rng(d)
    cot = rng.standard_normal((d, d)).astype(np.float32)
    gref = O.vjp(A64, cot.astype(np.float64), n, 0.0, 1.0, "sum", integrator)
    g = core.compute_vjp(n, A, cot, t0=0.0, tf=1.0, op="sum", integrator=integrator, precision="mixed",
                         checkpoint_K=32)
    assert rel(g, gref) <= 1e-6, rel(g, gref)


def test_mixed_long_four_element_problems_use_long_chunks(cuda):
    """Mixed-form 2x2 and SpaceCurve problems with >= 65537 samples run with
    1024-sample chunks by default (fewer FP64 scan steps); forward and VJP
    stay within 1e-6 of the FP64 oracle."""
    from magnus_gb300 import workloads
    S = 65537
    A = workloads.config0_samples(seed=5, d=2, samples=S)
    ref = O.forward(A, 5, 0.0, 1.0, "many", "Boole")
    out = core.compute(5, A, 0.0, 1.0, op="many", integrator="Boole", precision="mixed")
    for k in range(5):
        assert rel(out[k], ref[k]) <= 1e-6, (k, rel(out[k], ref[k]))
    cot = np.random.default_rng(5).standard_normal((2, 2))
    gref = O.vjp(A, cot, 5, 0.0, 1.0, "sum", "Boole")
    g = core.compute_vjp(5, A, cot, t0=0.0, tf=1.0, op="sum", integrator="Boole", precision="mixed")
    assert rel(g, gref) <= 1e-6, rel(g, gref)

    F = workloads.config1_samples_np(*workloads.config1_coeffs(seed=12, batch=1), samples=S, dtype=np.float64)[0]
    ref = O.forward_sc(F, 6, 0.0, 2.0, "many", "Simpson")
    out = core.compute_sc(6, F, 0.0, 2.0, op="many", integrator="Simpson", precision="mixed")
    scale = max(np.linalg.norm(r) for r in ref)
    for k in range(6):
        den = np.linalg.norm(ref[k]) if np.linalg.norm(ref[k]) >= 1e-6 * scale else scale
        assert np.linalg.norm(out[k] - ref[k]) / den <= 1e-6, k
    cot = np.random.default_rng(6).standard_normal((6, 3))
    gref = O.vjp_sc(F, cot, 6, 0.0, 2.0, "many", "Simpson")
    g = core.compute_sc_vjp(6, F, cot, t0=0.0, tf=2.0, op="many", integrator="Simpson", precision="mixed")
    assert rel(g, gref) <= 1e-6, rel(g, gref)


@pytest.mark.parametrize("integrator,S", [("Boole", 1025), ("Simpson", 1023), ("Trapezoid", 1023), ("Riemann", 1000)])
def test_mma32_scale_jumps(integrator, S, cuda, monkeypatch):
    """The d = 32 warp-MMA kernel predicts each operand's power-of-two scale
    from the previous group and re-splits when the prediction misses.  Here
    A(t) is zero on the first third of the samples, jumps to a scale 1e3
    larger on the middle third and back down: every operand (A, the prefixes
    P_j, the cotangents G_j) jumps by orders of magnitude between groups, in
    both directions, at chunk boundaries and inside chunks.  Every order stays
    within 1e-6; dA on this input is at the mixed form's own floor (about
    2.3e-6, as the FP32 SIMT kernel measures it), so the warp-MMA variants'
    dA is held to that kernel's error."""
    d, n = 32, 4
    A = smooth_samples(S, d, seed=77)
    A[: S // 3] = 0.0
    A[S // 3: 2 * S // 3] *= 1e3
    A = A.astype(np.float32)
    A64 = A.astype(np.float64)
    ref = O.forward(A64, n, 0.0, 1.0, "many", integrator)
    cot = np.random.default_rng(5).standard_normal((d, d)).astype(np.float32)
    gref = O.vjp(A64, cot.astype(np.float64), n, 0.0, 1.0, "sum", integrator)
    err = {}
    for variant in (0, 2, 3):
        monkeypatch.setenv("MGB_FORCE_VARIANT", str(variant))
        out = core.compute(n, A, 0.0, 1.0, op="many", integrator=integrator, precision="mixed", checkpoint_K=64)
        for k in range(n):
            assert rel(out[k], ref[k]) <= 1e-6, (variant, k, rel(out[k], ref[k]))
        g = core.compute_vjp(n, A, cot, t0=0.0, tf=1.0, op="sum", integrator=integrator, precision="mixed",
                             checkpoint_K=64)
        err[variant] = rel(g, gref)
    assert err[0] <= 5e-6, err
    assert err[2] <= 1.25 * err[0] + 1e-7 and err[3] <= 1.25 * err[0] + 1e-7, err


@pytest.mark.parametrize("d", [16, 32])
def test_scan_forms_agree(d, cuda, monkeypatch):
    """The mixed form's chunk scans at d = 16 / 32 run in double-FP32 and
    read the chunk kernels' transfer totals as FP32 pairs; MGB_DF_SCAN=0
    switches them to the FP64 scans (transfers stored in FP64).  Both agree
    with the oracle within 1e-6 per order and for dA."""
    A = smooth_samples(2049, d, seed=d + 11).astype(np.float32)
    A64 = A.astype(np.float64)
    n = 5
    ref = O.forward(A64, n, 0.0, 1.0, "many", "Boole")
    cot = np.random.default_rng(d).standard_normal((d, d)).astype(np.float32)
    gref = O.vjp(A64, cot.astype(np.float64), n, 0.0, 1.0, "sum", "Boole")
    for df in ("1", "0"):
        monkeypatch.setenv("MGB_DF_SCAN", df)
        out = core.compute(n, A, 0.0, 1.0, op="many", integrator="Boole", precision="mixed", checkpoint_K=64)
        for k in range(n):
            assert rel(out[k], ref[k]) <= 1e-6, (df, k, rel(out[k], ref[k]))
        g = core.compute_vjp(n, A, cot, t0=0.0, tf=1.0, op="sum", integrator="Boole", precision="mixed",
                             checkpoint_K=64)
        assert rel(g, gref) <= 1e-6, (df, rel(g, gref))
