"""CPU checks of the p-value stage's arithmetic schemes (hpdex_gb300/csrc/pvalue_math.cuh),
restated in exact rational arithmetic: every multiply / fma is rounded once to the nearest
double, as the device's __dmul_rn / __fma_rn do.

1. Divisions by a known reciprocal (Markstein's correction steps): tie sum / (N (N - 1)) from
   y = RN(1 / (N (N - 1))) and x / 12 from RN(1/12) must equal the correctly rounded quotient,
   on random operands, on the tie-sum / N(N - 1) operands of the p-value stage, and on quotients
   next to a rounding midpoint.
2. erfc from the table of Taylor coefficients at k / 128 (13 terms, Hermite recurrence) must
   stay within a few ulp of a 50-digit erfc.
The device implementation of both is checked on the GPU (hpdex_selftest_division,
hpdex_selftest_erfc)."""
import math
import random
from fractions import Fraction as F

import pytest


def rn(x):
    return float(x)  # int / int true division in CPython is correctly rounded (ties to even)


def mul(a, b):
    return rn(F(a) * F(b))


def fma(a, b, c):
    return rn(F(a) * F(b) + F(c))


def div_by_recip(a, b, y):
    q0 = mul(a, y)
    q1 = fma(fma(-b, q0, a), y, q0)
    return fma(fma(-b, q1, a), y, q1)


def div12(x):
    y = 0.083333333333333329
    q0 = mul(x, y)
    return fma(fma(-12.0, q0, x), y, q0)


def _cases(rng, n):
    for _ in range(n):
        kind = rng.randrange(3)
        if kind == 0:  # tie sums over N (N - 1)
            N = float(rng.randrange(2, 1 << 24))
            yield float(rng.getrandbits(rng.randrange(1, 54))), N * (N - 1.0)
        elif kind == 1:  # random doubles
            yield (math.ldexp(1.0 + rng.random(), rng.randrange(-60, 61)),
                   math.ldexp(1.0 + rng.random(), rng.randrange(-60, 61)))
        else:  # a / b next to the midpoint between q and its successor
            q = math.ldexp(1.0 + rng.random(), rng.randrange(-30, 31))
            b = math.ldexp(1.0 + rng.random(), rng.randrange(-30, 31))
            half_ulp = (math.nextafter(q, math.inf) - q) / 2
            yield fma(q, b, mul(half_ulp, b)), b


def test_divisions_by_known_reciprocal_are_correctly_rounded():
    rng = random.Random(7)
    assert F(0.083333333333333329) * 12 == 1 - F(1, 2 ** 54)  # RN(1/12) = (1 - 2^-54) / 12
    for a, b in _cases(rng, 6000):
        y = rn(F(1) / F(b))
        assert div_by_recip(a, b, y) == rn(F(a) / F(b)), (a, b)
        assert div12(a) == rn(F(a) / 12), a


def _erfc_table_step(x):
    """erfc(|x|) from the Taylor coefficients at the nearest k / 128, Horner with fmas."""
    ax = abs(x)
    k = round(ax * 128)
    xk = k / 128.0
    d = ax - xk
    E = 1.1283791670955126 * math.exp(-xk * xk)
    c = [math.erfc(xk)]
    hm1, h, fact, sign = 0.0, 1.0, 1.0, 1.0
    for n in range(1, 13):
        fact *= n
        c.append(-E * sign * h / fact)
        hm1, h = h, 2.0 * xk * h - 2.0 * (n - 1) * hm1
        sign = -sign
    r = c[12]
    for n in range(11, -1, -1):
        r = fma(r, d, c[n])
    return r


def test_erfc_taylor_table_scheme_matches_high_precision_erfc():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    rng = random.Random(3)
    xs = [rng.uniform(0.0, 6.0) for _ in range(1500)] + [rng.uniform(6.0, 26.0) for _ in range(500)]
    worst = 0.0
    for x in xs:
        ref = mpmath.erfc(mpmath.mpf(x))
        got = _erfc_table_step(x)
        worst = max(worst, float(abs((mpmath.mpf(got) - ref) / ref)))
    assert worst < 4e-15, worst
