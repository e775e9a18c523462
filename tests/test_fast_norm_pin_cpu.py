"""fast_norm=True: the oracle's restatement pinned to the reference's own scalar code.

The reference's fast normal tail lives in src/cpp/include/common.hpp: fast_erfc (Numerical
Recipes' erfcc), normal_sf, precompute_mu_inv_sd and p_asymptotic_{two_sided,greater,less}.
oracle/build_ref.sh compiles exactly those lines, unmodified, with the harness
oracle/ref_fast_scalar.cpp into oracle/_ref/libref_fast_scalar.so (only where the reference
sources are present). Here the oracle's oracle_p_asymptotic_fast, which the device's
p_asymptotic_fast is tested against on the GPU, must return the same doubles, bit for bit, on
seeded tests that cover all three alternatives, continuity on and off, tie sums up to the
all-tied maximum, the zero-variance and empty-group cases, and |U1 - mu| < cc (where the
reference's two-sided p exceeds 1 and is not clipped).

The reference's vectorised variant of the same polynomial (array_p_asymptotic_*, Highway)
nests the terms differently and cannot be built here (Highway is an empty submodule); it is
not covered.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import ROOT

LIB = os.path.join(ROOT, "oracle", "_ref", "libref_fast_scalar.so")


@pytest.fixture(scope="module")
def ref_fast():
    if not os.path.exists(LIB):
        pytest.skip("the reference's scalar fast_norm code was not built (sources absent)")
    L = ctypes.CDLL(LIB)
    L.ref_fast_p.restype = None
    L.ref_fast_p.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_double, ctypes.c_int,
                                                     ctypes.c_int64, ctypes.c_void_p]

    def run(U1, n1, n2, tie, cc, alt):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (U1, n1, n2, tie)]
        out = np.empty_like(arrs[0])
        L.ref_fast_p(*[a.ctypes.data for a in arrs], cc, alt, arrs[0].size, out.ctypes.data)
        return out
    return run


def _tests(seed, n=20_000):
    rng = np.random.default_rng(seed)
    n1 = np.exp(rng.uniform(0.0, np.log(60_000), n)).astype(np.int64).astype(np.float64)
    n2 = np.exp(rng.uniform(0.0, np.log(60_000), n)).astype(np.int64).astype(np.float64)
    n1[:50] = 0.0                       # empty reference: sigma 0, p = 1
    n1[50:100], n2[50:100] = 1.0, 1.0   # two observations
    nm = n1 * n2
    # half-integer U1 over [0, n1 n2], and U1 at mu +- a fraction of cc
    U1 = np.floor(rng.random(n) * (2 * nm + 1)) / 2
    U1[100:200] = 0.5 * nm[100:200] + rng.choice([-0.5, -0.25, 0.0, 0.25, 0.5], 100)
    N = n1 + n2
    full = N ** 3 - N                   # every value tied
    tie = np.floor(rng.random(n) ** 4 * full)
    tie[200:250] = full[200:250]        # all tied: zero variance
    return U1, n1, n2, tie


@pytest.mark.parametrize("alt", [0, 1, 2])
@pytest.mark.parametrize("cc", [0.0, 0.5])
def test_oracle_fast_norm_equals_reference_scalar_code(ref_fast, alt, cc):
    from oracle import oracle
    U1, n1, n2, tie = _tests(seed=17 + alt)
    want = ref_fast(U1, n1, n2, tie, cc, alt)
    got = oracle.p_asymptotic_fast(U1, n1, n2, tie, cc, alt)
    assert np.array_equal(got.view(np.int64), want.view(np.int64)), (
        int(np.sum(got != want)), float(np.max(np.abs(got - want))))


def test_reference_two_sided_fast_p_is_not_clipped(ref_fast):
    """|U1 - mu| < cc gives z < 0 and a two-sided p above 1 in the reference's scalar path."""
    p = ref_fast([50.0], [10.0], [10.0], [0.0], 0.5, 2)[0]
    assert p > 1.0
