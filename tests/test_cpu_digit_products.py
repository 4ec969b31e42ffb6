"""The arithmetic of the Cholesky's tensor-core trailing update (the Ozaki scheme),
restated in numpy and checked against exact rational arithmetic.

A panel column is scaled by a power of two and split into 8 signed digits (the first
within [-128, 128], the others within [-64, 64]); the digit-pair products of one
diagonal a + b = D, summed over K = 128, must stay below 2^24 so that an FP32
accumulator holds them exactly; the 36 pairs with a + b < 8 packed into one integer
V = sum_{D<6} S_D 2^(40-7D) + round((S_6 2^7 + S_7) / 2^9) must reproduce X^T X to
better than FP64 GEMM does (tolerance: 3e-16 of sqrt(G_ii G_jj), below the 1e-15 of
an FP64 dot product of length 128).
"""
from fractions import Fraction

import numpy as np
import pytest


def _digits(X, S=8):
    mx = np.abs(X).max(axis=0)
    e = np.where(mx > 0, np.frexp(mx)[1], 0)
    y = X / np.ldexp(1.0, e)[None, :]
    D = []
    for _ in range(S):
        t = y * 128.0
        d = np.rint(t)
        D.append(d)
        y = t - d
    return e, D


@pytest.mark.parametrize("seed", [0, 1])
def test_digit_products_reproduce_xtx(seed):
    rng = np.random.default_rng(seed)
    K, m = 128, 40
    X = rng.standard_normal((K, m)) * np.exp(rng.uniform(-25, 5, size=m))[None, :]
    X *= np.exp(rng.uniform(-4, 0, size=(K, m)))
    e, D = _digits(X)
    assert np.abs(D[0]).max() <= 128 and max(np.abs(d).max() for d in D[1:]) <= 64
    S = [sum(D[a].T @ D[Dg - a] for a in range(Dg + 1)) for Dg in range(8)]   # 0-based diagonals
    for s in S:   # every diagonal sum is an integer an FP32 accumulator holds exactly
        assert np.abs(s).max() < 2 ** 24
        assert np.array_equal(s.astype(np.float32).astype(np.float64), s)
    ref = X.astype(np.longdouble).T @ X.astype(np.longdouble)
    norm = np.sqrt(np.outer(np.diag(ref), np.diag(ref))).astype(np.float64)
    worst = 0.0
    for i in range(0, m, 3):
        for j in range(i, m, 2):
            Si = [int(S[d][i, j]) for d in range(8)]
            V = sum(Si[d] << (40 - 7 * d) for d in range(6)) + (((Si[6] << 7) + Si[7] + 256) >> 9)
            val = np.ldexp(float(V), int(e[i] + e[j] - 54))
            exact = sum(Fraction(float(X[k, i])) * Fraction(float(X[k, j])) for k in range(K))
            worst = max(worst, abs(float(Fraction(val) - exact)) / norm[i, j])
    fp64 = float(np.abs((X.T @ X - ref) / norm).max())
    print(f"\npacked digit products vs exact: {worst:.2e}; FP64 GEMM vs exact: {fp64:.2e}")
    assert worst <= 3e-16
