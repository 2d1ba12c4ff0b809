"""Complex matrix data on the GPU: the plain form against the reference's
complex128 outputs (forward, bilinear VJP, carry record), complex64 in the
mixed form against the complex128 run, and torch autograd on complex
tensors (conjugate-Wirtinger convention) against finite differences."""
import numpy as np
import pytest

import magnus_gb300 as magnus
from conftest import load_cases, rel

pytestmark = pytest.mark.gpu

CASES = load_cases("complex.npz")
core = magnus._core
KEYS = sorted(k for k in CASES if len(k) == 4 and k[0] == "c" and k[1:].isdigit())  # c000, c001, ...; not "c64"


@pytest.mark.parametrize("key", KEYS)
def test_complex128_matches_reference(key, cuda):
    c = CASES[key]
    out = core.compute(c["n"], c["A"], c["t0"], c["tf"], op=c["op"], integrator=c["integrator"], precision="plain")
    assert out.dtype == np.complex128 and out.shape == c["out"].shape
    assert rel(out, c["out"]) <= 1e-12, rel(out, c["out"])
    dA = core.compute_vjp(c["n"], c["A"], c["cot"], t0=c["t0"], tf=c["tf"], op=c["op"], integrator=c["integrator"],
                          precision="plain")
    assert dA.dtype == np.complex128 and dA.shape == c["A"].shape
    assert rel(dA, c["dA"]) <= 1e-12, rel(dA, c["dA"])


@pytest.mark.parametrize("key", sorted(k for k in CASES if k.startswith("carry")))
def test_complex_carry_record_matches_reference(key, cuda):
    c = CASES[key]
    out, carry = core.compute(c["n"], c["A"], c["t0"], c["tf"], op=c["op"], integrator=c["integrator"],
                              record_vjp=True, precision="plain")
    assert rel(out, c["out"]) <= 1e-12
    assert carry.shape == c["carry"].shape
    assert rel(carry, c["carry"]) <= 1e-12, rel(carry, c["carry"])


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_complex64_against_complex128(precision, cuda):
    c = CASES["c64"]
    out = core.compute(c["n"], c["A"], c["t0"], c["tf"], op=c["op"], integrator=c["integrator"], precision=precision)
    assert out.dtype == np.complex64
    for k in range(int(c["n"])):
        assert rel(out[k], c["out64"][k]) <= 2e-6, (k, rel(out[k], c["out64"][k]))


def test_complex_autograd_matches_finite_differences(cuda):
    import torch
    from magnus_gb300.autograd import magnus as magnus_t
    rng = np.random.default_rng(5)
    S, d, n = 33, 3, 4
    A = torch.tensor((rng.standard_normal((S, d, d)) + 1j * rng.standard_normal((S, d, d))) / np.sqrt(2 * d),
                     device=cuda, requires_grad=True)
    W = torch.tensor(rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d)), device=cuda)

    def loss(X):
        return (magnus_t(X, n, 0.0, 1.0, op="sum", integrator="Boole") * W).real.sum()

    loss(A).backward()
    g = A.grad
    V = torch.tensor(rng.standard_normal((S, d, d)) + 1j * rng.standard_normal((S, d, d)), device=cuda)
    eps = 1e-6
    with torch.no_grad():
        fd = (loss(A + eps * V) - loss(A - eps * V)) / (2 * eps)
    # for a real loss, dL = Re <conj(grad), dA> with torch's convention
    pred = (g.conj() * V).real.sum()
    assert abs(float(fd) - float(pred)) <= 1e-7 * max(1.0, abs(float(fd))), (float(fd), float(pred))


@pytest.mark.parametrize("key", sorted(k for k in CASES if k.startswith("z")))
def test_complex128_spacecurve_matches_reference(key, cuda):
    c = CASES[key]
    out = core.compute_sc(c["n"], c["A"], c["t0"], c["tf"], op=c["op"], integrator=c["integrator"],
                          precision="plain")
    assert out.dtype == np.complex128 and out.shape == c["out"].shape
    assert rel(out, c["out"]) <= 1e-12, rel(out, c["out"])
    dA = core.compute_sc_vjp(c["n"], c["A"], c["cot"], t0=c["t0"], tf=c["tf"], op=c["op"],
                             integrator=c["integrator"], precision="plain")
    assert dA.dtype == np.complex128 and dA.shape == c["A"].shape
    assert rel(dA, c["dA"]) <= 1e-12, rel(dA, c["dA"])


@pytest.mark.parametrize("key", sorted(k for k in CASES if k.startswith("sccarry")))
def test_complex_spacecurve_carry_matches_reference(key, cuda):
    c = CASES[key]
    out, carry = core.compute_sc(c["n"], c["A"], c["t0"], c["tf"], op=c["op"], integrator=c["integrator"],
                                 record_vjp=True, precision="plain")
    assert rel(out, c["out"]) <= 1e-12
    assert carry.shape == c["carry"].shape
    assert rel(carry, c["carry"]) <= 1e-12, rel(carry, c["carry"])
