"""The blocked Gauss-Jordan inverse of the dense coarsest level, restated in
numpy (the arithmetic of ples_gb300/csrc/gauss_jordan.cuh, not its code).

Column by column, step c picks the unused row p_c with the largest |K(r, c)|
(ties to the lowest row) and takes row r -= f_r row p_c, f_r = K(r, c) /
K(p_c, c), in K and in S, whose column c starts as the unit vector of p_c.
The blocked form runs a panel's steps on the panel's K columns only, keeps
the multipliers F, and applies the product T of the panel's eliminations to
every other column at once: T v = v - F w with w = L^-1 v(p), L(c, c') =
F(p_c, c') below the diagonal.  Both give the same pivots and the inverse
(row c of the inverse = row p_c of S over K(p_c, c), column order by pivot).
"""
import numpy as np
import pytest


def _pivot(col, used):
    cand = np.where(used, 0.0, np.abs(col))
    p = int(np.argmax(cand))  # the first of equal maxima: the lowest row
    assert cand[p] > 0.0, "singular"
    return p


def _extract(K, S, piv):
    m = K.shape[0]
    inv = np.empty_like(K)
    for c in range(m):
        r = piv[c]
        inv[c, piv] = S[r, :] / K[r, c]
    return inv


def column_by_column(K0):
    K, m = K0.copy(), K0.shape[0]
    S = np.zeros_like(K)
    used = np.zeros(m, bool)
    piv = np.zeros(m, int)
    for c in range(m):
        p = _pivot(K[:, c], used)
        used[p], piv[c] = True, p
        S[p, c] = 1.0
        f = K[:, c] / K[p, c]
        f[p] = 0.0
        K[:, c + 1:] -= np.outer(f, K[p, c + 1:])
        S[:, :c + 1] -= np.outer(f, S[p, :c + 1])
    return _extract(K, S, piv), piv


def blocked(K0, B):
    K, m = K0.copy(), K0.shape[0]
    S = np.zeros_like(K)
    used = np.zeros(m, bool)
    piv = np.zeros(m, int)
    for c0 in range(0, m, B):
        nb = min(B, m - c0)
        c1 = c0 + nb
        P = K[:, c0:c1].copy()
        F = np.zeros((m, nb))
        for c in range(nb):  # the panel's steps on its own columns
            p = _pivot(P[:, c], used)
            used[p], piv[c0 + c] = True, p
            f = P[:, c] / P[p, c]
            f[p] = 0.0
            P[:, c + 1:] -= np.outer(f, P[p, c + 1:])
            F[:, c] = f
        K[:, c0:c1] = P
        S[piv[c0:c1], np.arange(c0, c1)] = 1.0
        V = np.concatenate([S[:, :c1], K[:, c1:]], axis=1)  # column d: S below c1, K from c1
        L = F[piv[c0:c1], :]
        W = np.zeros((nb, m))
        for c in range(nb):
            W[c] = V[piv[c0 + c]] - L[c, :c] @ W[:c]
        V -= F @ W
        S[:, :c1], K[:, c1:] = V[:, :c1], V[:, c1:]
    return _extract(K, S, piv), piv


@pytest.mark.parametrize("m,B", [(37, 16), (37, 8), (64, 16), (5, 16)])
def test_blocked_inverse_matches_column_by_column_and_numpy(m, B):
    rng = np.random.default_rng(m * 100 + B)
    K = rng.uniform(-1.0, 1.0, (m, m))
    K[np.arange(0, m, 3), np.arange(0, m, 3)] = 0.0  # zero diagonals force row exchanges
    ref = np.linalg.inv(K)
    inv_c, piv_c = column_by_column(K)
    inv_b, piv_b = blocked(K, B)
    assert np.array_equal(piv_c, piv_b)
    scale = np.abs(ref).max()
    assert np.abs(inv_c - ref).max() <= 1e-10 * scale
    assert np.abs(inv_b - ref).max() <= 1e-10 * scale


def test_blocked_inverse_of_a_bordered_singular_operator():
    """The coarsest system's shape: a periodic 1-D Laplacian (singular, with
    constant null vector) bordered by [[M, v], [1^T, 0]] is invertible; the
    blocked inverse solves it."""
    n = 21
    M = np.zeros((n, n))
    for i in range(n):
        M[i, i] = -2.0
        M[i, (i + 1) % n] = M[i, (i - 1) % n] = 1.0
    K = np.zeros((n + 1, n + 1))
    K[:n, :n] = M
    K[:n, n] = 1.0
    K[n, :n] = 1.0
    inv_b, _ = blocked(K, 8)
    assert np.abs(inv_b @ K - np.eye(n + 1)).max() <= 1e-10
