"""Collapsed FP64 restatement of the reference's Magnus recursion, in numpy —
TEST INFRASTRUCTURE ONLY (the checker for full-size configurations).

The C oracle (magnus_oracle.c) restates the reference's per-Gauss-Legendre-
node recursion literally: Q (n - 1) products per sample, single-threaded.  At
the benchmarked sizes (d = 32..128, S = 16385..65537) that takes minutes per
instance.  This module computes the same quantities in FP64 with the nodes
collapsed (n - 1 products per sample, batched matrix products), and is pinned
against the C oracle on every rule and op by tests/test_collapsed_cpu.py.

Forward (src/magnus.hpp:12-261 restated; the collapse: prefix is linear and
commutes with right-multiplication by a constant):
    W_1 = A,  P_j = prefix(W_j),  T_j = P_j[S-1],  W_{j+1}[i] = A[i] P_j[i]
    per GL node x_q (s = x_q - 1): D_1 = I, D_m = s sum_{j<m} T_j D_{m-j}
    E_m = sum_q w_q D_m,  Omega_1 = T_1,  Omega_k = sum_{j<=k} T_j E_{k-j+1}
Adjoint (src/grad.hpp:59-349 restated): tau_j = dL/dT_j through the small
algebra, then, for j = n..1,
    P-bar_j = tau_j at sample S-1 + A^T W-bar_{j+1},  W-bar_j = prefix^T(P-bar_j)
    dA = W-bar_1 + sum_j W-bar_{j+1} P_j^T.

The prefix rules are evaluated with cumulative sums over rule blocks:
    Boole     src/integration/boole.hpp:24-74
    Simpson   src/integration/simpson.hpp:24-58
    Trapezoid src/integration/trapezoid.hpp:23-33
    Riemann   src/integration/default.hpp:23-26 (inclusive)
and prefix^T is their exact transpose (boole.hpp:108-151, simpson.hpp:77-100,
trapezoid.hpp:43-50, default.hpp:32-38 compute the same map in place).
Matrix data only (SpaceCurve and 2 x 2 problems are cheap for the C oracle).
"""
from __future__ import annotations

import numpy as np

# Block length B and the partial-rule weights (in units of dt) for the sample
# r = 1..B positions after a block anchor: P[b + r] = P[b] + dt * w_r . f[b..b+r].
_BLOCKS = {
    "Boole": (4, {1: [1 / 2, 1 / 2], 2: [1 / 3, 4 / 3, 1 / 3], 3: [3 / 8, 9 / 8, 9 / 8, 3 / 8],
                  4: [14 / 45, 64 / 45, 24 / 45, 64 / 45, 14 / 45]}),
    "Simpson": (2, {1: [1 / 2, 1 / 2], 2: [1 / 3, 4 / 3, 1 / 3]}),
    "Trapezoid": (1, {1: [1 / 2, 1 / 2]}),
}


def gl_nodes(n):
    """Nodes and weights of the Q = (n+3)/2 point Gauss-Legendre rule on
    [0, 1] (src/util/gen_nodes.py:20-27; Q = 1 for n = 1)."""
    Q = (n + 3) // 2 if n > 1 else 1
    x, w = np.polynomial.legendre.leggauss(Q)
    return (x + 1) / 2, w / 2


def prefix(f, dt, rule):
    """Cumulative rule integral P (same shape as f, axis 0 = samples)."""
    S = f.shape[0]
    if rule == "Riemann":
        return dt * np.cumsum(f, axis=0)
    B, w = _BLOCKS[rule]
    if (S - 1) % B:
        raise ValueError("sample interval count violates integrator divisibility")
    nb = (S - 1) // B
    F = f.reshape(S, -1)
    Fb = F[:B * nb].reshape(nb, B, -1)  # block k, positions 0..B-1
    Fe = F[B::B]                         # block k, position B (the next anchor)
    P = np.zeros_like(F)
    Pb = P[:B * nb].reshape(nb, B, -1)
    inc = dt * (np.tensordot(np.array(w[B][:B]), Fb, axes=(0, 1)) + w[B][B] * Fe)
    anchors = np.concatenate([np.zeros_like(F[:1]), np.cumsum(inc, axis=0)])  # P at b = 0, B, 2B, ...
    Pb[:, 0] = anchors[:nb]
    P[S - 1] = anchors[nb]
    for r in range(1, B):
        Pb[:, r] = anchors[:nb] + dt * np.tensordot(np.array(w[r]), Fb[:, :r + 1], axes=(0, 1))
    return P.reshape(f.shape)


def prefix_t(H, dt, rule):
    """prefix^T: G[k] = sum_i R[i, k] H[i] for the rule's prefix matrix R."""
    S = H.shape[0]
    if rule == "Riemann":
        return dt * np.cumsum(H[::-1], axis=0)[::-1]
    B, w = _BLOCKS[rule]
    nb = (S - 1) // B
    Hf = H.reshape(S, -1)
    Hb = Hf[:B * nb].reshape(nb, B, -1)
    He = Hf[B::B]
    G = np.zeros_like(Hf)
    Gb = G[:B * nb].reshape(nb, B, -1)
    # cotangent on block k's increment from every later block's samples
    # (their values all include the anchor the increment feeds)
    hb = Hb[:, 1:].sum(axis=1) + He
    later = np.concatenate([np.cumsum(hb[::-1], axis=0)[::-1][1:], np.zeros_like(hb[:1])])
    He = He + later
    for r in range(1, B + 1):
        Hr = He if r == B else Hb[:, r]
        for s, c in enumerate(w[r]):
            if s < B:
                Gb[:, s] += (c * dt) * Hr
            else:
                G[B::B] += (c * dt) * Hr
    return G.reshape(H.shape)


def _small_forward(T, n):
    """Omega_1..Omega_n, E and the per-node D from the totals T_1..T_n."""
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


def _small_adjoint(T, E, Ds, Obar, n):
    """tau_j = dL/dT_j given Omega-bar (the adjoint of _small_forward)."""
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


def _levels(A, n, dt, rule):
    P, W = [], A
    for j in range(n):
        Pj = prefix(W, dt, rule)
        P.append(Pj)
        if j + 1 < n:
            W = np.matmul(A, Pj)
    return P


def _apply_op(Om, op, n):
    if op == "many":
        return np.stack(Om)
    if op == "sum":
        return sum(Om)
    return Om[n - 1]


def orders(A, n, t0=0.0, tf=1.0, integrator="Boole"):
    """Omega_1..Omega_n as an (n, d, d) FP64 array (op 'many')."""
    A = np.asarray(A, dtype=np.float64)
    dt = (tf - t0) / (A.shape[0] - 1)
    T = [Pj[-1] for Pj in _levels(A, n, dt, integrator)]
    return np.stack(_small_forward(T, n)[0])


def forward(A, n, t0=0.0, tf=1.0, op="sum", integrator="Boole"):
    """The reference's compute(...) output for matrix data, in FP64."""
    return _apply_op(list(orders(A, n, t0, tf, integrator)), op, n)


def vjp(A, cot, n, t0=0.0, tf=1.0, op="sum", integrator="Boole"):
    """The reference's compute_vjp(...) dA for matrix data, in FP64."""
    A = np.asarray(A, dtype=np.float64)
    cot = np.asarray(cot, dtype=np.float64)
    S, d = A.shape[0], A.shape[1]
    dt = (tf - t0) / (S - 1)
    P = _levels(A, n, dt, integrator)
    T = [Pj[-1] for Pj in P]
    _, E, Ds = _small_forward(T, n)
    zero = np.zeros((d, d))
    Obar = [cot[k] if op == "many" else (cot if (op == "sum" or k == n - 1) else zero) for k in range(n)]
    tau = _small_adjoint(T, E, Ds, Obar, n)
    At = np.swapaxes(A, 1, 2)
    dA = np.zeros_like(A)
    Wbar = None
    for j in range(n, 0, -1):
        Pbar = np.zeros_like(A) if Wbar is None else np.matmul(At, Wbar)
        Pbar[-1] += tau[j - 1]
        if Wbar is not None:
            dA += np.matmul(Wbar, np.swapaxes(P[j - 1], 1, 2))
        P[j - 1] = None  # release the level once used
        Wbar = prefix_t(Pbar, dt, integrator)
    dA += Wbar
    return dA
