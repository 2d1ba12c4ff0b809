"""Executable statement, in numpy, of the algorithm the GPU kernels implement,
checked against the oracle (the reference's per-node recursion) on the CPU:

* the Gauss-Legendre node collapse: n - 1 products per sample
  (W_1 = A, P_j = prefix(W_j), W_{j+1} = A P_j, T_j = P_j[S-1]) and the small
  algebra D^(q), E, Omega in FP64;
* the chunked form: zero-carry local levels per chunk, chunk transfers
  Lambda^c_j and the scan pi^{c+1}_j = pi^c_j + Lambda^c_j +
  sum_{m<j} Lambda^c_{j-m} pi^c_m (Chen's identity);
* the adjoint: tau_j from the small algebra, then P-bar_j = tau_j at the last
  sample + A^T W-bar_{j+1}, W-bar_j = prefix^T(P-bar_j),
  dA = W-bar_1 + sum_j W-bar_{j+1} P_j^T;
* the mixed form's step dt_k (rule weights exact in FP32) and the rescaling
  of level j by (dt/dt_k)^j;
* SpaceCurves as the associative quaternion recursion with signed levels.

The block rules are stated as explicit (S x S) prefix matrices, so prefix^T is
their transpose.  Reference rules: src/integration/boole.hpp:24-74,
simpson.hpp:24-58, trapezoid.hpp:23-33, default.hpp:23-26; the per-node
recursion: src/magnus.hpp:60-84, src/grad.hpp:149-349.
"""
import numpy as np
import pytest

import oracle as O

RULES = ["Boole", "Simpson", "Trapezoid", "Riemann"]


def prefix_matrix(S, dt, rule):
    """R (S x S) with P[i] = sum_k R[i, k] f[k] for the rule's prefix."""
    R = np.zeros((S, S))
    if rule == "Riemann":  # inclusive: P_i = dt sum_{k <= i} f_k
        for i in range(S):
            R[i, :i + 1] = dt
        return R
    if rule == "Trapezoid":
        for i in range(1, S):
            R[i] = R[i - 1]
            R[i, i - 1] += dt / 2
            R[i, i] += dt / 2
        return R
    if rule == "Simpson":
        for i in range(1, S):
            if i % 2 == 1:  # P_i = P_{i-1} + dt/2 (f_{i-1} + f_i)
                R[i] = R[i - 1]
                R[i, i - 1] += dt / 2
                R[i, i] += dt / 2
            else:           # P_i = P_{i-2} + dt/3 (f_{i-2} + 4 f_{i-1} + f_i)
                R[i] = R[i - 2]
                R[i, i - 2:i + 1] += dt / 3 * np.array([1.0, 4.0, 1.0])
        return R
    # Boole: within each block of 4 from the last anchor b (a multiple of 4)
    w = {1: np.array([1.0, 1.0]) * dt / 2, 2: np.array([1.0, 4.0, 1.0]) * dt / 3,
         3: np.array([1.0, 3.0, 3.0, 1.0]) * 3 * dt / 8, 4: np.array([14.0, 64.0, 24.0, 64.0, 14.0]) * dt / 45}
    for i in range(1, S):
        b = ((i - 1) // 4) * 4
        R[i] = R[b]
        R[i, b:i + 1] += w[i - b]
    return R


def gl_nodes(n):
    Q = (n + 3) // 2 if n > 1 else 1
    x, w = np.polynomial.legendre.leggauss(Q)
    return (x + 1) / 2, w / 2


def levels(A, n, R):
    """P_1..P_n (S, d, d) by the collapsed recursion."""
    P = []
    W = A
    for j in range(n):
        Pj = np.einsum("ik,kab->iab", R, W)
        P.append(Pj)
        W = A @ Pj
    return P


def small_forward(T, n):
    """Omega_1..Omega_n from the totals T_1..T_n (FP64 small algebra)."""
    d = T[0].shape[0]
    x, w = gl_nodes(n)
    E = [np.zeros((d, d)) for _ in range(n)]
    Ds = []
    for xq, wq in zip(x, w):
        s = xq - 1.0
        D = [np.eye(d)]
        for m in range(2, n + 1):
            D.append(s * sum(T[j - 1] @ D[m - j - 1] for j in range(1, m)))
        Ds.append(D)
        for m in range(n):
            E[m] += wq * D[m]
    Om = [T[0]] + [sum(T[j - 1] @ E[k - j] for j in range(1, k + 1)) for k in range(2, n + 1)]
    return Om, E, Ds


def small_adjoint(T, E, Ds, Obar, n):
    """tau_j = dL/dT_j given Omega-bar (the adjoint of small_forward)."""
    d = T[0].shape[0]
    x, w = gl_nodes(n)
    tau = [np.zeros((d, d)) for _ in range(n)]
    Ebar = [np.zeros((d, d)) for _ in range(n)]
    tau[0] += Obar[0]
    for k in range(2, n + 1):
        for j in range(1, k + 1):
            tau[j - 1] += Obar[k - 1] @ E[k - j].T
            Ebar[k - j] += T[j - 1].T @ Obar[k - 1]
    for (xq, wq), D in zip(zip(x, w), Ds):
        s = xq - 1.0
        Dbar = [wq * Ebar[m] for m in range(n)]
        for m in range(n, 1, -1):
            for j in range(1, m):
                tau[j - 1] += s * Dbar[m - 1] @ D[m - j - 1].T
                Dbar[m - j - 1] += s * T[j - 1].T @ Dbar[m - 1]
    return tau


def collapsed_forward(A, n, t0, tf, rule):
    S = A.shape[0]
    R = prefix_matrix(S, (tf - t0) / (S - 1), rule)
    T = [Pj[-1] for Pj in levels(A, n, R)]
    return np.array(small_forward(T, n)[0])


def chunked_totals(A, n, t0, tf, rule, K):
    """T_1..T_n from chunk-local levels and the scan over chunk transfers."""
    S, d = A.shape[0], A.shape[1]
    dt = (tf - t0) / (S - 1)
    pi = [np.zeros((d, d)) for _ in range(n)]  # pi_1..pi_n at the chunk start (pi_0 = I)
    b = 0
    while b < S - 1:
        e = min(b + K, S - 1)
        if rule == "Riemann" and b > 0:
            idx = np.arange(b + 1, e + 1)  # inclusive rule: the shared sample belongs to the earlier chunk
            Rl = prefix_matrix(len(idx) + 1, dt, "Riemann")[1:, 1:]
        else:
            idx = np.arange(b, e + 1)
            Rl = prefix_matrix(len(idx), dt, rule)
        Al = A[idx]
        # local levels: L_0 = I, L_k = prefix_loc(A L_{k-1})
        L = [np.broadcast_to(np.eye(d), Al.shape)]
        for k in range(n):
            L.append(np.einsum("ik,kab->iab", Rl, Al @ L[-1]))
        lam = [L[j][-1] for j in range(1, n + 1)]  # Lambda_j = L_j at the chunk end
        pi = [pi[j - 1] + lam[j - 1] + sum(lam[j - m - 1] @ pi[m - 1] for m in range(1, j)) for j in range(1, n + 1)]
        b = e
    return pi


@pytest.mark.parametrize("rule", RULES)
def test_node_collapse_equals_per_node_recursion(rule):
    rng = np.random.default_rng(1)
    S = 65 if rule != "Riemann" else 60
    A = rng.standard_normal((S, 3, 3)) / np.sqrt(3)
    ref = O.forward(A, 5, 0.0, 1.0, "many", rule)
    out = collapsed_forward(A, 5, 0.0, 1.0, rule)
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) <= 1e-13


@pytest.mark.parametrize("K", [4, 8, 24])
@pytest.mark.parametrize("rule", RULES)
def test_chunked_scan_equals_whole_prefix(rule, K):
    rng = np.random.default_rng(2)
    S = 65 if rule != "Riemann" else 61
    A = rng.standard_normal((S, 2, 2)) / np.sqrt(2)
    R = prefix_matrix(S, 1.0 / (S - 1), rule)
    T = [Pj[-1] for Pj in levels(A, 4, R)]
    Tc = chunked_totals(A, 4, 0.0, 1.0, rule, K)
    for j in range(4):
        assert np.linalg.norm(Tc[j] - T[j]) <= 1e-13 * max(1.0, np.linalg.norm(T[j]))


@pytest.mark.parametrize("op", ["one", "many", "sum"])
@pytest.mark.parametrize("rule", RULES)
def test_adjoint_equals_reference_vjp(rule, op):
    rng = np.random.default_rng(3)
    S, d, n = (33 if rule != "Riemann" else 30), 3, 4
    A = rng.standard_normal((S, d, d)) / np.sqrt(d)
    cot = rng.standard_normal((n, d, d) if op == "many" else (d, d))
    R = prefix_matrix(S, 1.0 / (S - 1), rule)
    P = levels(A, n, R)
    T = [Pj[-1] for Pj in P]
    _, E, Ds = small_forward(T, n)
    Obar = [cot[k] if op == "many" else (cot if (op == "sum" or k == n - 1) else np.zeros((d, d)))
            for k in range(n)]
    tau = small_adjoint(T, E, Ds, Obar, n)
    # reverse over levels: P-bar_j = tau_j e_{S-1} + A^T W-bar_{j+1}; W-bar_j = R^T P-bar_j
    dA = np.zeros_like(A)
    Wbar_next = None
    for j in range(n, 0, -1):
        Pbar = np.zeros_like(A)
        Pbar[-1] += tau[j - 1]
        if Wbar_next is not None:
            Pbar += np.swapaxes(A, 1, 2) @ Wbar_next
            dA += Wbar_next @ np.swapaxes(P[j - 1], 1, 2)
        Wbar_next = np.einsum("ki,kab->iab", R, Pbar)
    dA += Wbar_next
    ref = O.vjp(A, cot, n, 0.0, 1.0, op, rule)
    assert np.linalg.norm(dA - ref) / np.linalg.norm(ref) <= 1e-12


@pytest.mark.parametrize("rule,u", [("Boole", 90.0), ("Simpson", 6.0), ("Trapezoid", 2.0), ("Riemann", 1.0)])
def test_mixed_step_rescaling(rule, u):
    """The mixed form integrates with dt_k = u 2^round(log2(dt/u)) (every rule
    weight dt_k c/u exact in FP32) and rescales the totals by
    (dt/dt_k)^j: level j is homogeneous of degree j in the step."""
    rng = np.random.default_rng(4)
    S = 33 if rule != "Riemann" else 30
    A = rng.standard_normal((S, 2, 2))
    dt = 0.7 / (S - 1)
    dtk = u * 2.0 ** np.round(np.log2(dt / u))
    for c in {"Boole": [1 / 2, 1 / 3, 3 / 8, 9 / 8, 4 / 3, 14 / 45, 64 / 45, 24 / 45], "Simpson": [1 / 2, 1 / 3, 4 / 3],
              "Trapezoid": [1 / 2], "Riemann": [1.0]}[rule]:
        w = dtk * c
        assert np.float32(w) == w  # exact in FP32
    T = [Pj[-1] for Pj in levels(A, 4, prefix_matrix(S, dt, rule))]
    Tk = [Pj[-1] for Pj in levels(A, 4, prefix_matrix(S, dtk, rule))]
    sig = dt / dtk
    for j in range(4):
        assert np.allclose(Tk[j] * sig ** (j + 1), T[j], rtol=1e-13, atol=1e-15 * np.abs(T[j]).max())


def test_spacecurve_product_is_negated_quaternion_product():
    """The reference's SpaceCurve product c = (a.b, -b0 a + a x b) on padded
    (0, a) equals -qmul(a, b), qmul(a, b) = b (x) a (Hamilton), so the
    recursion runs on the associative qmul with level signs (-1)^(k-1)."""
    rng = np.random.default_rng(5)

    def hamilton(p, q):
        p0, pv, q0, qv = p[0], p[1:], q[0], q[1:]
        return np.concatenate([[p0 * q0 - pv @ qv], p0 * qv + q0 * pv + np.cross(pv, qv)])

    for _ in range(20):
        a = np.concatenate([[0.0], rng.standard_normal(3)])
        b = rng.standard_normal(4)
        ref_c = np.concatenate([[a[1:] @ b[1:]], -b[0] * a[1:] + np.cross(a[1:], b[1:])])
        assert np.allclose(ref_c, -hamilton(b, a), atol=1e-14)
    # the whole recursion: SpaceCurve data through the oracle equals the
    # associative recursion on qmul with signed outputs
    F = rng.standard_normal((33, 3)) * 0.5
    n = 4
    ref = O.forward_sc(F, n, 0.0, 1.0, "many", "Boole")
    S = F.shape[0]
    R = prefix_matrix(S, 1.0 / (S - 1), "Boole")
    A4 = np.concatenate([np.zeros((S, 1)), F], axis=1)
    P, W = [], A4
    for _ in range(n):
        Pj = R @ W
        P.append(Pj)
        W = np.array([hamilton(p, a) for a, p in zip(A4, Pj)])  # qmul(a, p) = p (x) a
    # qmul-algebra small forward: represent quaternions by their 4x4 right-multiplication matrices
    def rmat(q):
        return np.array([hamilton(np.eye(4)[k], q) for k in range(4)]).T  # x -> x (x) q
    T = [rmat(Pj[-1]) for Pj in P]
    Om, _, _ = small_forward(T, n)
    for k in range(n):
        q = Om[k] @ np.eye(4)[0]  # the quaternion itself: 1 (x) q
        sign = (-1) ** k
        assert np.allclose(sign * q[1:], ref[k], rtol=1e-12, atol=1e-13 * np.abs(ref).max())
