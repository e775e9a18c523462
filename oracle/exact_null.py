"""Exact null distribution of the Mann-Whitney U statistic in Python integers.

TEST INFRASTRUCTURE ONLY (oracle for the GPU exact-mode tables).

The number of arrangements of m reference and n target observations (no ties) whose U
equals u is the coefficient of q^u in the Gaussian binomial [m+n choose m]_q =
prod_{i=1..m} (1 - q^(n+i)) / (1 - q^i). The survival P(U >= u) is the tail sum divided by
C(m+n, m), rounded once to float64. This is the null scipy.stats.mannwhitneyu(method=
"exact") uses (scipy/stats/_mannwhitneyu.py, class _MWU), with the same statistic choice:
two-sided -> 2 * sf(floor(max(U1, U2))), greater -> sf(floor(U1)), less -> sf(floor(U2)),
clipped to [0, 1].
"""
from __future__ import annotations

from fractions import Fraction
from functools import lru_cache
from math import comb, floor


@lru_cache(maxsize=256)
def mwu_counts(m: int, n: int) -> tuple:
    """Integer counts f(u) for u = 0..m*n."""
    top = m * n
    poly = [0] * (top + 1)
    poly[0] = 1
    for i in range(1, m + 1):
        # multiply by (1 - q^(n+i))
        s = n + i
        for u in range(top, s - 1, -1):
            poly[u] -= poly[u - s]
        # divide by (1 - q^i): running sum with stride i (exact)
        for u in range(i, top + 1):
            poly[u] += poly[u - i]
    return tuple(poly)


@lru_cache(maxsize=256)
def mwu_tails(m: int, n: int) -> tuple:
    """Integer tail sums sum_{v >= u} f(v) for u = 0..m*n."""
    f = mwu_counts(m, n)
    out = [0] * len(f)
    s = 0
    for u in range(len(f) - 1, -1, -1):
        s += f[u]
        out[u] = s
    return tuple(out)


def mwu_sf_exact(u: float, m: int, n: int) -> float:
    """P(U >= floor(u)) under the null, as the correctly rounded float64 of the fraction."""
    k = floor(u)
    if k <= 0:
        return 1.0
    if k > m * n:
        return 0.0
    return float(Fraction(mwu_tails(m, n)[k], comb(m + n, m)))


def p_exact(U1: float, m: int, n: int, alternative: int) -> float:
    """alternative: 0 less, 1 greater, 2 two-sided (the reference's enum)."""
    if m * n == 0:
        return 1.0
    U2 = m * n - U1
    if alternative == 2:
        p = 2.0 * mwu_sf_exact(max(U1, U2), m, n)
    elif alternative == 1:
        p = mwu_sf_exact(U1, m, n)
    else:
        p = mwu_sf_exact(U2, m, n)
    return min(max(p, 0.0), 1.0)
