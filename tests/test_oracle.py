"""Pins the CPU oracle (oracle/mwu_oracle.c) to the reference's own outputs.

Every fixture under tests/golden/ was produced by the reference's compiled kernel
(AI4Cell/hpdex src/cpp/module.cpp + mannwhitneyu.cpp, built by oracle/build_ref.sh) on the
stored inputs; the oracle must reproduce U1 and P bit for bit, the same error text, and the
group means of both summation modes exactly.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference_fixture(name, oracle_lib):
    g = load_golden(name)
    o = g["options"]
    args = (g["data"], g["indices"], g["indptr"], g["group_id"], g["n_targets"])
    if g["error"]:
        with pytest.raises(RuntimeError) as e:
            oracle_lib.mannwhitneyu(*args, tie_correction=o["tie_correction"],
                                    use_continuity=o["use_continuity"],
                                    zero_handling=o["zero_handling"],
                                    alternative=o["alternative"], method=o["method"], threads=2)
        assert str(e.value) == g["error"]
    else:
        U1, P = oracle_lib.mannwhitneyu(*args, tie_correction=o["tie_correction"],
                                        use_continuity=o["use_continuity"],
                                        zero_handling=o["zero_handling"],
                                        alternative=o["alternative"], method=o["method"],
                                        threads=2)
        np.testing.assert_array_equal(U1, g["U1"])
        np.testing.assert_array_equal(P, g["P"])
    G = g["n_targets"] + 1
    for include_zeros, sfx in ((True, ""), (False, "_nz")):
        plain = oracle_lib.group_mean(*args[:4], G, include_zeros, 2, False)
        kahan = oracle_lib.group_mean(*args[:4], G, include_zeros, 2, True)
        np.testing.assert_array_equal(plain, g["mean_plain" + sfx])
        np.testing.assert_array_equal(kahan, g["mean_kahan" + sfx])


def test_oracle_asymptotic_matches_scipy(oracle_lib):
    """FP64 scipy semantics (scipy.stats.mannwhitneyu on float64 copies) for the three
    alternatives with and without continuity, on the small_float fixture's genes."""
    stats = pytest.importorskip("scipy.stats")
    g = load_golden("small_float")
    import scipy.sparse as sp
    X = sp.csc_matrix((g["data"], g["indices"], g["indptr"]),
                      shape=(g["group_id"].size, g["indptr"].size - 1)).toarray().astype(np.float64)
    gid = g["group_id"]
    T = g["n_targets"]
    for alt_i, alt in enumerate(("less", "greater", "two-sided")):
        for cont in (False, True):
            U1, P = oracle_lib.mannwhitneyu(g["data"], g["indices"], g["indptr"], gid, T,
                                            use_continuity=cont, zero_handling=3,
                                            alternative=alt_i, threads=2)
            for c in range(0, X.shape[1], 37):
                for t in range(1, T + 1):
                    r = stats.mannwhitneyu(X[gid == 0, c], X[gid == t, c], alternative=alt,
                                           method="asymptotic", use_continuity=cont)
                    i = c * T + (t - 1)
                    assert U1[i] == r.statistic
                    assert abs(P[i] - r.pvalue) <= 1e-13 * max(r.pvalue, 1e-300)


def test_oracle_exact_reference_discrepancy(oracle_lib):
    """The reference's exact p counts bounded compositions, not the MWU null: for n1=5,
    n2=4, U=12 its survival is 0.32224 (two-sided 0.64448), while the exact MWU null gives
    P(U>=12) = 23/63 = 0.365079... (two-sided 0.730158..., what scipy reports)."""
    sf = oracle_lib.p_exact_reference(12.0, 5, 4)
    assert abs(sf - 0.32224) < 1e-15
    from oracle.exact_null import mwu_sf_exact
    assert abs(2 * mwu_sf_exact(12, 5, 4) - 0.7301587301587301) < 1e-15


def test_exact_null_matches_scipy_exact():
    """The exact-integer MWU null (oracle/exact_null.py) against scipy's exact mode on tie-free
    samples of the exact configuration's shapes (reference of up to 40, targets of 3-40):
    x = reference, y = target, so scipy's statistic is U1."""
    from scipy.stats import mannwhitneyu
    from oracle.exact_null import p_exact
    rng = np.random.default_rng(5)
    names = {0: "less", 1: "greater", 2: "two-sided"}
    for m, n in [(40, 3), (40, 17), (40, 40), (12, 30), (7, 5), (1, 9)]:
        for _ in range(4):
            z = rng.permutation(m + n).astype(np.float64)
            x, y = z[:m], z[m:]
            for alt, name in names.items():
                r = mannwhitneyu(x, y, alternative=name, method="exact")
                ours = p_exact(float(r.statistic), m, n, alt)
                assert abs(ours - r.pvalue) <= 1e-12 * max(r.pvalue, 1e-300), (m, n, alt)


def test_oracle_fast_norm_path_restates_reference_scalar_form():
    """fast_norm: Numerical Recipes erfcc (fractional error < 1.2e-7 of erfc), the reference's
    own arithmetic for mu and 1/sigma, and no clip of the two-sided p (|U1 - mu| < cc gives a
    p above 1, as in the reference's scalar path)."""
    import math
    from oracle import oracle
    rng = np.random.default_rng(0)
    n1 = rng.integers(5, 400, 500).astype(np.float64)
    n2 = rng.integers(5, 400, 500).astype(np.float64)
    U1 = np.floor(rng.random(500) * n1 * n2)
    tie = np.zeros(500)
    for alt in (0, 1, 2):
        pf = oracle.p_asymptotic_fast(U1, n1, n2, tie, 0.5, alt)
        pp = np.array([oracle.lib().oracle_p_asymptotic(u, a, b, 0.0, 0.5, alt)
                       for u, a, b in zip(U1, n1, n2)])
        ok = pp > 1e-12
        assert np.all(np.abs(pf[ok] - pp[ok]) <= 3e-7 * np.maximum(pp[ok], 1e-2))
    p = oracle.p_asymptotic_fast([50.0], [10.0], [10.0], [0.0], 0.5, 2)[0]
    assert p > 1.0 and math.isclose(p, 1.0301501, rel_tol=1e-6)
