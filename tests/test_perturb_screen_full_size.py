"""The benchmark workload at full size, through the CUDA path.

perturb_screen: 200,000 cells x 8,000 genes, 1.47e8 stored float32 values, 20,000 reference
cells and 500 targets, i.e. 4e6 tests. The oracle runs the whole workload in a few seconds on
the host cores, so every test is compared with it. Properties that hold at any size are
checked beside it.

Bars:
- U1 bit-exact, and P within 1e-12 relative (absolute floor 1e-300) of the oracle. This covers
  the public one-shot call (chunked upload pipeline) and a resident plan (persistent kernel,
  fused p-values, CUDA graph) in every zero mode and alternative run here.
- 2 U1 is an integer, 0 <= U1 <= n1 n2, and P lies in [0, 1].
- The two-sided p equals twice the one-sided p of the larger U side, clipped at 1, bit for bit.
  The reference computes both from the same z.
- zero_handling='none' raises the oracle's error text: sparse genes leave too few explicit
  values.
- Group means (include_zeros) match the oracle within 1e-10 relative. Both are sums of at most
  200,000 positive doubles, so each is within 2e-11 of the exact sum.

Collected after the test_gpu_* files.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P_RTOL = 1e-12
P_FLOOR = 1e-300
ALT = {0: "less", 1: "greater", 2: "two-sided"}
ZH = {0: "none", 1: "min", 2: "max", 3: "mix"}


@pytest.fixture(scope="module")
def screen():
    from hpdex_gb300 import synthetic
    w = synthetic.perturb_screen()
    assert (w.n_rows, w.n_cols, w.n_targets) == (200_000, 8_000, 500)
    return w


@pytest.fixture(scope="module")
def oracle_results(screen):
    """Oracle (U1, P) per (zero_handling, alternative), target-major (T, C), computed once."""
    from oracle import oracle
    cache = {}

    def get(zh, alt):
        if (zh, alt) not in cache:
            w = screen
            U1, P = oracle.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                        tie_correction=True, use_continuity=True,
                                        zero_handling=zh, alternative=alt, method=2, threads=-1)
            cache[(zh, alt)] = (U1.reshape(w.n_cols, w.n_targets).T,
                                P.reshape(w.n_cols, w.n_targets).T)
        return cache[(zh, alt)]
    return get


@pytest.fixture(scope="module")
def resident(screen):
    from hpdex_gb300.resident import ResidentMatrix
    w = screen
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    yield M
    M.close()


def group_sizes(w):
    """n1 (reference) and n2 per target: every assigned cell counts in min/max/mix."""
    g = w.group_id
    sizes = np.bincount(g[(g >= 0) & (g <= w.n_targets)], minlength=w.n_targets + 1)
    return float(sizes[0]), sizes[1:].astype(np.float64)


def assert_p_close(P, Pref):
    bad = np.abs(P - Pref) > np.maximum(P_RTOL * np.abs(Pref), P_FLOOR)
    if bad.any():
        err = np.abs(P - Pref) / np.maximum(np.abs(Pref), P_FLOOR)
        raise AssertionError(f"{int(bad.sum())} p-values off, max rel err {err.max():.3e}")


def assert_statistics(w, U1, P):
    n1, n2 = group_sizes(w)
    nm = (n1 * n2)[:, None]
    assert np.all(2.0 * U1 == np.round(2.0 * U1))
    assert np.all((U1 >= 0) & (U1 <= nm))
    assert np.all((P >= 0.0) & (P <= 1.0))


def plan_results(M, w, zh, alt):
    from hpdex_gb300.resident import BATCHED
    plan = M.plan(w.group_id, w.n_targets, zero_handling=ZH[zh], alternative=ALT[alt],
                  use_continuity=True, tie_correction=True)
    try:
        plan.run(BATCHED)
        return plan.download()
    finally:
        plan.close()


def test_public_call_matches_oracle(screen, oracle_results):
    from hpdex_gb300.backend.bin import kernel
    w = screen
    U1, P = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                tie_correction=True, use_continuity=True, zero_handling=1,
                                alternative=2, fast_norm=False)
    U1o, Po = oracle_results(1, 2)
    assert U1.shape == (w.n_targets, w.n_cols)
    np.testing.assert_array_equal(U1, U1o)
    assert_p_close(P, Po)
    assert_statistics(w, U1, P)


@pytest.mark.parametrize("zh,alt", [(1, 2), (1, 1), (1, 0), (2, 2), (3, 2)])
def test_resident_plan_matches_oracle(screen, oracle_results, resident, zh, alt):
    w = screen
    U1, P = plan_results(resident, w, zh, alt)
    U1o, Po = oracle_results(zh, alt)
    np.testing.assert_array_equal(U1, U1o)
    assert_p_close(P, Po)
    assert_statistics(w, U1, P)


def test_two_sided_is_twice_the_larger_side(screen, resident):
    w = screen
    U1, P2 = plan_results(resident, w, 1, 2)
    _, Pl = plan_results(resident, w, 1, 0)
    _, Pg = plan_results(resident, w, 1, 1)
    n1, n2 = group_sizes(w)
    U2 = (n1 * n2)[:, None] - U1
    one_sided = np.where(U1 >= U2, Pg, Pl)
    np.testing.assert_array_equal(P2, np.minimum(1.0, 2.0 * one_sided))


def test_none_mode_raises_the_oracle_error(screen):
    from oracle import oracle
    from hpdex_gb300.backend.bin import kernel
    w = screen
    with pytest.raises(RuntimeError) as eo:
        oracle.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                            zero_handling=0, use_continuity=True, threads=-1)
    with pytest.raises(RuntimeError) as eg:
        kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                            zero_handling=0, use_continuity=True, fast_norm=False)
    assert str(eg.value) == str(eo.value)


def test_group_means_match_oracle(screen):
    from oracle import oracle
    from hpdex_gb300.backend.bin import kernel
    w = screen
    G = w.n_targets + 1
    m = kernel.group_mean(w.data, w.indices, w.indptr, w.group_id, G, include_zeros=True)
    mo = oracle.group_mean(w.data, w.indices, w.indptr, w.group_id, G, include_zeros=True)
    np.testing.assert_allclose(m, mo, rtol=1e-10, atol=0.0)


def test_ranking_of_p_and_fdr_matches_oracle(screen, oracle_results, resident):
    """All 4e6 tests ranked by P (stable argsort) in the same order as the oracle's P, and the
    device's BH FDR of its own P ranking them as scipy's BH of the oracle's P does."""
    from scipy.stats import false_discovery_control
    from hpdex_gb300._lib import bh_fdr
    w = screen
    _, P = plan_results(resident, w, 1, 2)
    _, Po = oracle_results(1, 2)
    p, po = P.reshape(-1), np.ascontiguousarray(Po).reshape(-1)
    np.testing.assert_array_equal(np.argsort(p, kind="stable"), np.argsort(po, kind="stable"))
    fdr, fdr_o = bh_fdr(p), false_discovery_control(po, method="bh")
    np.testing.assert_array_equal(np.argsort(fdr, kind="stable"), np.argsort(fdr_o, kind="stable"))
