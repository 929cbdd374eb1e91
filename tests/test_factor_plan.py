"""The block plans of the rebuild's recursive factorisations
(dynemol_gb300/csrc/elhl_api.cu: tri_inverse / tri_inverse_top / trmm_*_oop,
chol_inv_df), replayed on the host with the block constants read from the
source: every leaf is a diagonal block of the expected size, the leaves tile
the matrix, and no block exceeds the workspace factor_workspace allocates
(ld x (ld / 2 + kTriBlock) elements).  A numpy replay of the same splits
checks the algorithms on small matrices."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = open(os.path.join(ROOT, "dynemol_gb300", "csrc", "elhl_api.cu")).read()
LEAF = 64       # leaf_rows(): 64-row diagonal blocks (factor.cu)
CHOL_SPLIT = 64  # chol_inv_df splits on multiples of 64


def _const(name):
    m = re.search(r"constexpr int %s = (\d+);" % name, SRC)
    assert m, name
    return int(m.group(1))


TRI_BLOCK, TRMM_LEAF = _const("kTriBlock"), _const("kTrmmLeaf")


def ru(x, m):
    return (x + m - 1) // m * m


def workspace(ld):
    assert "cs.ld * (cs.ld / 2 + kTriBlock)" in SRC
    return ld * (ld // 2 + TRI_BLOCK)


def tri_plan(n, ld):
    """Largest workspace use of tri_inverse, and the top-down leaves."""
    need = 0
    s = LEAF
    while s < TRI_BLOCK:
        npairs, rem = n // (2 * s), n - 2 * s * (n // (2 * s))
        need = max(need, npairs * s * s, (rem - s) * s if rem > s else 0)
        s *= 2
    leaves = []

    def top(a, m):
        nonlocal need
        if m <= TRI_BLOCK:
            leaves.append((a, m))
            return
        n1 = ru(m // 2, TRI_BLOCK)
        assert 0 < n1 < m
        need = max(need, ld * n1)
        top(a, n1)
        top(a + n1, m - n1)

    top(0, n)
    return need, leaves


def chol_plan(n, ld):
    need, leaves = 0, []

    def rec(a, m):
        nonlocal need
        if m <= LEAF:
            leaves.append((a, m))
            return
        n1 = ru(m // 2, CHOL_SPLIT)
        assert 0 < n1 < m
        need = max(need, ld * n1)
        rec(a, n1)
        rec(a + n1, m - n1)

    rec(0, n)
    return need, leaves


@pytest.mark.parametrize("n", list(range(1, 600)) + list(range(600, 4097, 7)) + [2170, 3720, 8192, 16384])
def test_plans_fit_the_workspace(n):
    ld = ru(n, 32)
    w = workspace(ld)
    for plan, block in ((tri_plan, TRI_BLOCK), (chol_plan, LEAF)):
        need, leaves = plan(n, ld)
        assert need <= w, (plan.__name__, n, need, w)
        # leaves tile [0, n) with aligned blocks of at most `block` rows
        pos = 0
        for a, m in leaves:
            assert a == pos and a % block == 0 and 0 < m <= block
            pos += m
        assert pos == n


def _tri_inverse(L):
    """G = L^-1 by the splits of tri_inverse (bottom-up batched pairs, then
    top-down with both triangular products as full products of the blocks)."""
    n = L.shape[0]
    A = L.copy()
    for r in range(0, n, LEAF):
        b = slice(r, min(n, r + LEAF))
        A[b, b] = np.linalg.inv(A[b, b])
    s = LEAF
    while s < TRI_BLOCK:
        for o in range(0, n - s, 2 * s):
            e = min(n, o + 2 * s)
            i1, i2 = slice(o, o + s), slice(o + s, e)
            A[i2, i1] = -A[i2, i2] @ (A[i2, i1] @ A[i1, i1])
        s *= 2

    def top(a, m):
        if m <= TRI_BLOCK:
            return
        n1 = ru(m // 2, TRI_BLOCK)
        top(a, n1)
        top(a + n1, m - n1)
        i1, i2 = slice(a, a + n1), slice(a + n1, a + m)
        A[i2, i1] = -A[i2, i2] @ (A[i2, i1] @ A[i1, i1])

    top(0, n)
    return A


def _chol_inv(S):
    n = S.shape[0]
    A, G = np.tril(S).copy(), np.zeros_like(S)

    def rec(a, m):
        i = slice(a, a + m)
        if m <= LEAF:
            Lb = np.linalg.cholesky(A[i, i] + np.tril(A[i, i], -1).T)
            A[i, i], G[i, i] = Lb, np.linalg.inv(Lb)
            return
        n1 = ru(m // 2, CHOL_SPLIT)
        i1, i2 = slice(a, a + n1), slice(a + n1, a + m)
        rec(a, n1)
        A[i2, i1] = A[i2, i1] @ G[i1, i1].T
        A[i2, i2] -= np.tril(A[i2, i1] @ A[i2, i1].T)
        rec(a + n1, m - n1)
        G[i2, i1] = -G[i2, i2] @ (A[i2, i1] @ G[i1, i1])

    rec(0, n)
    return np.tril(A), np.tril(G)


@pytest.mark.parametrize("n", [1, 63, 64, 65, 130, 300, 513, 700, 1100])
def test_plans_compute_the_factors(n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, n))
    S = X @ X.T / n + np.eye(n)
    L = np.linalg.cholesky(S)
    G = _tri_inverse(L)
    assert np.abs(np.tril(G) - np.linalg.inv(L)).max() < 1e-12
    L2, G2 = _chol_inv(S)
    assert np.abs(L2 - L).max() < 1e-12
    assert np.abs(G2 - np.linalg.inv(L)).max() < 1e-12
