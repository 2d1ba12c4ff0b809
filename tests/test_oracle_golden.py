"""The CPU oracle (oracle/magnus_oracle.c) against the reference's own outputs
stored in tests/golden (generated by tests/golden/make_golden.py from the
reference compiled from source).  Bar: <= 1e-13 relative Frobenius."""
import numpy as np
import pytest

import oracle as O
from conftest import load_cases, rel

SMALL = load_cases("small.npz")
MEDIUM = load_cases("medium.npz")


def _run_case(c):
    if c["kind"] == "matrix":
        out = O.forward(c["A"], c["n"], c["t0"], c["tf"], c["op"], c["integrator"])
        dA = O.vjp(c["A"], c["cot"], c["n"], c["t0"], c["tf"], c["op"], c["integrator"]) if "cot" in c else None
    else:
        out = O.forward_sc(c["A"], c["n"], c["t0"], c["tf"], c["op"], c["integrator"])
        dA = O.vjp_sc(c["A"], c["cot"], c["n"], c["t0"], c["tf"], c["op"], c["integrator"]) if "cot" in c else None
    return out, dA


@pytest.mark.parametrize("key", sorted(SMALL))
def test_oracle_small_cases(key):
    c = SMALL[key]
    out, dA = _run_case(c)
    assert out.shape == c["out"].shape
    assert rel(out, c["out"]) <= 1e-13
    assert rel(dA, c["dA"]) <= 1e-13


@pytest.mark.parametrize("key", sorted(MEDIUM))
def test_oracle_medium_cases(key):
    c = MEDIUM[key]
    out, dA = _run_case(c)
    assert rel(out, c["out"]) <= 1e-13
    assert rel(dA, c["dA"]) <= 1e-13


def test_oracle_carry_layout_matches_reference():
    checked = 0
    for c in SMALL.values():
        if "carry" not in c:
            continue
        if c["kind"] == "matrix":
            _, carry = O.forward(c["A"], c["n"], c["t0"], c["tf"], c["op"], c["integrator"], record_vjp=True)
        else:
            _, carry = O.forward_sc(c["A"], c["n"], c["t0"], c["tf"], c["op"], c["integrator"], record_vjp=True)
        assert carry.shape == c["carry"].shape
        assert rel(carry, c["carry"]) <= 1e-13
        # the reference's VJP consuming its own carry equals recomputation
        checked += 1
    assert checked >= 8


def test_oracle_config0():
    cases = load_cases("config0.npz")
    for c in cases.values():
        out = O.forward(c["A"], c["n"], c["t0"], c["tf"], c["op"], c["integrator"])
        assert rel(out, c["out"]) <= 1e-13


def test_oracle_float32_follows_reference_float32():
    c = load_cases("float32.npz")["f32"]
    out32 = O.forward(c["A"], c["n"], c["t0"], c["tf"], c["op"], c["integrator"])
    out64 = O.forward(c["A"].astype(np.float64), c["n"], c["t0"], c["tf"], c["op"], c["integrator"])
    assert out32.dtype == np.float32
    assert rel(out32, c["out"]) <= 1e-6
    assert rel(out64, c["out64"]) <= 1e-13


def test_oracle_vjp_with_carry_equals_recompute():
    rng = np.random.default_rng(5)
    A = rng.standard_normal((21, 3, 3)) / 2
    out, carry = O.forward(A, 5, 0.0, 1.0, "many", "Boole", record_vjp=True)
    cot = rng.standard_normal(out.shape)
    a = O.vjp(A, cot, 5, 0.0, 1.0, "many", "Boole", carry=carry)
    b = O.vjp(A, cot, 5, 0.0, 1.0, "many", "Boole")
    assert rel(a, b) <= 1e-14


def test_oracle_batch_threads_match_serial():
    rng = np.random.default_rng(6)
    A = rng.standard_normal((5, 33, 2, 2))
    cot = rng.standard_normal((5, 2, 2))
    fwd = O.batch(A, 4, 0.0, 1.0, "many", "Boole", threads=3)
    vjp = O.batch(A, 4, 0.0, 1.0, "sum", "Boole", cot=cot, threads=2)
    for b in range(5):
        np.testing.assert_array_equal(fwd[b].reshape(4, 2, 2), O.forward(A[b], 4, 0.0, 1.0, "many", "Boole"))
        np.testing.assert_array_equal(vjp[b].reshape(33, 2, 2),
                                      O.vjp(A[b], cot[b], 4, 0.0, 1.0, "sum", "Boole"))


def _embed(Z):
    """Complex (..., d, d) -> real (..., 2d, 2d) [[X, -Y], [Y, X]]."""
    X, Y = Z.real, Z.imag
    return np.concatenate([np.concatenate([X, -Y], -1), np.concatenate([Y, X], -1)], -2)


def test_complex_embedding_reproduces_reference():
    """The GB300 engine runs a complex d x d problem as the real 2d x 2d
    problem on [[Re A, -Im A], [Im A, Re A]], with the cotangent
    [[Re C, Im C], [-Im C, Re C]] / 2 and dA = (dR11 + dR22) + i (dR12 - dR21).
    Checked here with the oracle on the embedded problems against the
    reference's complex128 outputs (forward, bilinear VJP, carry record)."""
    cases = load_cases("complex.npz")
    for key, c in cases.items():
        if key == "c64" or c["kind"] != "matrix":
            continue
        A, n, op, integ = c["A"], int(c["n"]), str(c["op"]), str(c["integrator"])
        d = A.shape[-1]
        AR = _embed(A)
        outR = O.forward(AR, n, float(c["t0"]), float(c["tf"]), op, integ)
        out = outR[..., :d, :d] + 1j * outR[..., d:, :d]
        assert rel(out, c["out"]) <= 1e-13, key
        if "dA" in c:
            C = c["cot"]
            RC = np.concatenate([np.concatenate([C.real, C.imag], -1), np.concatenate([-C.imag, C.real], -1)], -2) / 2
            dR = O.vjp(AR, RC, n, float(c["t0"]), float(c["tf"]), op, integ)
            G = (dR[:, :d, :d] + dR[:, d:, d:]) + 1j * (dR[:, :d, d:] - dR[:, d:, :d])
            assert rel(G, c["dA"]) <= 1e-13, key


# e_s (x) e_c = SGN[s][c] e_IDX[s][c] (Hamilton, basis 1, i, j, k)
_IDX = [[0, 1, 2, 3], [1, 0, 3, 2], [2, 3, 0, 1], [3, 2, 1, 0]]
_SGN = [[1, 1, 1, 1], [1, -1, 1, -1], [1, -1, -1, 1], [1, 1, -1, -1]]


def _rho(a):
    """Right multiplication y -> y (x) a as a 4 x 4 (complex) matrix."""
    M = np.zeros((4, 4), dtype=complex)
    for s in range(4):
        for c in range(4):
            M[_IDX[s][c], s] += _SGN[s][c] * a[c]
    return M


def test_complex_spacecurve_embedding_reproduces_reference():
    """Complex SpaceCurve data run as the real 8 x 8 matrix problem (op many)
    on the embedding of rho(0, f); order k carries the sign (-1)^(k-1) and an
    element is the first column of its rho.  Checked with the oracle against
    the reference's complex128 SpaceCurve outputs and bilinear VJPs."""
    cases = load_cases("complex.npz")
    for key, c in cases.items():
        if c["kind"] != "spacecurve" or "dA" not in c:
            continue
        F, n, op, integ = c["A"], int(c["n"]), str(c["op"]), str(c["integrator"])
        t0, tf = float(c["t0"]), float(c["tf"])
        AR = np.stack([_embed(_rho(np.concatenate([[0], f]))) for f in F])
        M = O.forward(AR, n, t0, tf, "many", integ)
        Om = np.array([(M[k, :4, 0] + 1j * M[k, 4:, 0]) * (-1) ** k for k in range(n)])[:, 1:]
        got = Om if op == "many" else (Om.sum(0) if op == "sum" else Om[-1])
        assert rel(got, c["out"]) <= 1e-13, key
        C = c["cot"]
        RC = []
        for k in range(n):
            Ck = C[k] if op == "many" else (C if (op == "sum" or k == n - 1) else np.zeros(3))
            K = np.zeros((4, 4), dtype=complex)
            K[1:, 0] = (-1) ** k * Ck
            RC.append(np.concatenate([np.concatenate([K.real, K.imag], -1), np.concatenate([-K.imag, K.real], -1)],
                                     -2) / 2)
        dR = O.vjp(AR, np.stack(RC), n, t0, tf, "many", integ)
        G = (dR[:, :4, :4] + dR[:, 4:, 4:]) + 1j * (dR[:, :4, 4:] - dR[:, 4:, :4])
        da = np.zeros((len(F), 4), dtype=complex)
        for cc in range(4):
            for s in range(4):
                da[:, cc] += _SGN[s][cc] * G[:, _IDX[s][cc], s]
        assert rel(da[:, 1:], c["dA"]) <= 1e-13, key
