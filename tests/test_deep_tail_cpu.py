"""CPU checks of the deep tail of the p-values (|z| beyond ~37, p below 1e-300 and subnormal).

1. The oracle against the reference's own outputs on the strongly shifted workload
   (tests/golden/extreme_shift_outputs.npz, written by make_golden.py from the reference's
   compiled kernel): U1 and P bit for bit, for all three alternatives. Both call the host C
   library's erfc, so their subnormal p-values agree exactly.
2. The deep-tail steps of the device's erfc (erfc_tail in hpdex_gb300/csrc/pvalue_math.cuh),
   restated with IEEE doubles (Python floats round to nearest, subnormals included; fma
   through exact rationals), against the host C library's erfc on [26.5, 27.3]: equal below
   1e-311, where the subnormal grid is coarse; within one grid step and 1e-12 relative above.
The device itself is checked against the same library on the GPU (tests/test_gpu_deep_tail.py).
"""
import ctypes
import ctypes.util
import math
import os
import random
import struct
from fractions import Fraction as F

import numpy as np
import pytest

from conftest import GOLDEN

SMALLEST_NORMAL = 2.2250738585072014e-308


def libm_erfc():
    lib = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    lib.erfc.restype = ctypes.c_double
    lib.erfc.argtypes = [ctypes.c_double]
    return lib.erfc


def workload_digest(w):
    import hashlib
    h = hashlib.sha256()
    for a in (w.data, w.indices.astype(np.int64), w.indptr.astype(np.int64),
              w.group_id.astype(np.int32)):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@pytest.fixture(scope="module")
def extreme():
    from hpdex_gb300 import synthetic
    w = synthetic.extreme_shift()
    z = np.load(os.path.join(GOLDEN, "extreme_shift_outputs.npz"))
    assert str(z["digest"]) == workload_digest(w), "extreme_shift() no longer reproduces its inputs"
    return w, z


def test_fixture_reaches_the_subnormal_tail(extreme):
    _, z = extreme
    P = z["P_alt2"]
    assert ((P > 0) & (P < SMALLEST_NORMAL)).sum() >= 40
    assert (P == 0).sum() >= 100


@pytest.mark.parametrize("alt", [0, 1, 2])
def test_oracle_equals_reference_in_the_deep_tail(extreme, oracle_lib, alt):
    w, z = extreme
    U1, P = oracle_lib.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                    tie_correction=True, use_continuity=True, zero_handling=1,
                                    alternative=alt, method=2, threads=-1)
    np.testing.assert_array_equal(U1, z[f"U1_alt{alt}"])
    np.testing.assert_array_equal(P, z[f"P_alt{alt}"])


def _fma(a, b, c):
    return float(F(a) * F(b) + F(c))


def _high_word_only(x):
    b = struct.unpack("<Q", struct.pack("<d", x))[0] & 0xFFFFFFFF00000000
    return struct.unpack("<d", struct.pack("<Q", b))[0]


LN2_HI = float.fromhex("0x1.62e42fefa4000p-1")
LN2_LO = float.fromhex("-0x1.8432a1b0e2634p-43")
K_HI = float.fromhex("0x1.faf956cc3bebcp-1")
K_LO = float.fromhex("-0x1.b02ab54640020p-60")


def erfc_tail(ax):
    """erfc_tail of pvalue_math.cuh, step by step (math.exp stands in for the device's exp)."""
    z = _high_word_only(ax)
    a = (-z * z) - 0.5625
    if not a >= -750.0:
        return 0.0
    k = round(a * 1.4426950408889634)
    r = _fma(-float(k), LN2_HI, a) - float(k) * LN2_LO
    e1 = (math.exp(r) * 2.0 ** (k + 64)) * 2.0 ** -64
    u = 0.5 / (ax * ax)
    h = _fma(-15.0, u, 1.0)
    for n in range(13, 2, -2):
        h = _fma(-float(n) * u, h, 1.0)
    q = -u * h
    d = (ax - z) * (ax + z)
    t = _fma(-d, 0.2, 1.0)
    t = _fma(-d * 0.25, t, 1.0)
    t = _fma(-d / 3.0, t, 1.0)
    t = _fma(-d * 0.5, t, 1.0)
    p = -d * t
    g = _fma(q, p, q + p)
    f_lo = _fma(K_HI, g, K_LO)
    E = e1 * 2.0 ** 64
    ph = E * K_HI
    pl = _fma(E, K_HI, -ph)
    prod = (ph + _fma(E, f_lo, pl)) * 2.0 ** -64
    return prod / ax


def test_tail_constants():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    ln2 = mpmath.log(2)
    assert F(LN2_HI).denominator <= 2 ** 40  # 40 significant bits: k * hi is exact for |k| < 2^13
    assert abs(mpmath.mpf(LN2_HI) + mpmath.mpf(LN2_LO) - ln2) < mpmath.mpf(2) ** -95
    K = mpmath.exp(mpmath.mpf(9) / 16) / mpmath.sqrt(mpmath.pi)
    assert abs(mpmath.mpf(K_HI) + mpmath.mpf(K_LO) - K) < mpmath.mpf(2) ** -110


def test_tail_steps_equal_the_c_library():
    erfc = libm_erfc()
    rng = random.Random(11)
    xs = [rng.uniform(26.5, 27.3) for _ in range(20_000)] + [26.5, 27.226, 27.23, 27.5, 28.0, 40.0]
    deep_mismatch = 0
    for x in xs:
        ref, got = erfc(x), erfc_tail(x)
        if ref == got:
            continue
        if ref < 1e-311:
            deep_mismatch += 1
        assert abs(got - ref) <= max(1e-12 * ref, 5e-324), (x, ref, got)
    assert deep_mismatch == 0
