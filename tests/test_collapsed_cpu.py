"""Pins the collapsed FP64 checker (oracle/collapsed.py) against the C oracle
(the reference's per-node recursion restated) on every rule and op, and
against the reference's own outputs at config4's size, so that the
full-size GPU parity tests can use it where the C oracle would take minutes
per instance."""
import numpy as np
import pytest

import collapsed as Cl
import oracle as O
from conftest import load_cases, rel
from magnus_gb300 import workloads

RULES = [("Boole", 129), ("Simpson", 131), ("Trapezoid", 97), ("Riemann", 90)]


@pytest.mark.parametrize("op", ["one", "many", "sum"])
@pytest.mark.parametrize("rule,S", RULES)
@pytest.mark.parametrize("d,n", [(3, 5), (8, 4), (5, 1), (4, 2)])
def test_collapsed_checker_equals_oracle(rule, S, op, d, n):
    rng = np.random.default_rng(d * 100 + S + n)
    A = rng.standard_normal((S, d, d)) / np.sqrt(d)
    cot = rng.standard_normal((n, d, d) if op == "many" else (d, d))
    assert rel(Cl.forward(A, n, 0.2, 1.7, op, rule), O.forward(A, n, 0.2, 1.7, op, rule)) <= 1e-13
    assert rel(Cl.vjp(A, cot, n, 0.2, 1.7, op, rule), O.vjp(A, cot, n, 0.2, 1.7, op, rule)) <= 1e-13


def test_collapsed_checker_on_a_config4_shaped_instance():
    """d = 32, n = 5, Boole, float32-valued samples of the config4 form at
    S = 1025: forward per order and VJP within 1e-13 of the C oracle."""
    from magnus_gb300 import workloads
    Ck = workloads.config4_coeffs(seed=40, batch=1, d=32)
    A = workloads.config4_samples_np(Ck, samples=1025, dtype=np.float32)[0].astype(np.float64)
    ref = O.forward(A, 5, 0.0, 1.0, "many", "Boole")
    out = Cl.forward(A, 5, 0.0, 1.0, "many", "Boole")
    for k in range(5):
        assert rel(out[k], ref[k]) <= 1e-13, (k, rel(out[k], ref[k]))
    cot = workloads.config4_cotangent(batch=1, d=32)[0]
    assert rel(Cl.vjp(A, cot, 5, 0.0, 1.0, "sum", "Boole"), O.vjp(A, cot, 5, 0.0, 1.0, "sum", "Boole")) <= 1e-13


@pytest.mark.parametrize("rule,S", RULES)
def test_prefix_transpose_is_the_adjoint(rule, S):
    """<prefix(f), h> == <f, prefix^T(h)> for random f, h."""
    rng = np.random.default_rng(S)
    f = rng.standard_normal((S, 2, 3))
    h = rng.standard_normal((S, 2, 3))
    lhs = np.sum(Cl.prefix(f, 0.01, rule) * h)
    rhs = np.sum(f * Cl.prefix_t(h, 0.01, rule))
    assert abs(lhs - rhs) <= 1e-13 * max(1.0, abs(lhs))


def test_collapsed_checker_matches_reference_at_config4_size():
    """The FP64 checker the full-size GPU parity tests use, against the
    reference itself at config4's size (tests/golden/config4_full.npz: the
    reference's every order and its dA at 39 sample indices for one d = 32,
    S = 32769, n = 5 Boole trajectory with platform-independent samples)."""
    g = load_cases("config4_full.npz")["c4full"]
    n, S, d = int(g["n"]), int(g["samples"]), int(g["dim"])
    A64 = workloads.config4_poly_samples(seed=int(g["seed"]), samples=S, d=d)
    out = Cl.forward(A64, n, 0.0, 1.0, "many", "Boole")
    for k in range(n):
        assert rel(out[k], g["out"][k]) <= 1e-12, (k, rel(out[k], g["out"][k]))
    dA = Cl.vjp(A64, g["cot"], n, 0.0, 1.0, "sum", "Boole")
    idx = g["idx"]
    assert rel(dA[idx], g["dA_rows"]) <= 1e-12, rel(dA[idx], g["dA_rows"])
    assert abs(np.linalg.norm(dA) / g["dA_norm"] - 1.0) <= 1e-12


def test_collapsed_checker_matches_reference_at_config2_size():
    """As above at config2's size (tests/golden/config2_full.npz: one
    skew-symmetric d = 64, S = 16385, n = 4 Boole trajectory)."""
    g = load_cases("config2_full.npz")["c2full"]
    n, S, d = int(g["n"]), int(g["samples"]), int(g["dim"])
    A64 = workloads.config2_poly_samples(seed=int(g["seed"]), samples=S, d=d)
    out = Cl.forward(A64, n, 0.0, 1.0, "many", "Boole")
    for k in range(n):
        assert rel(out[k], g["out"][k]) <= 1e-12, (k, rel(out[k], g["out"][k]))
    dA = Cl.vjp(A64, g["cot"], n, 0.0, 1.0, "sum", "Boole")
    assert rel(dA[g["idx"]], g["dA_rows"]) <= 1e-12, rel(dA[g["idx"]], g["dA_rows"])
