"""GPU: p-values computed inside the rank kernel (fused, the default for asymptotic plans) equal
the separate p-value kernel's bit for bit, in both launch forms, and match the oracle.

The fused stage finishes each gene's tests during the CTA's next gene, and the CTA's last gene
after its work queue runs dry; a gene without stored elements (an empty column) leaves the
previous gene's tests to all warps. The workloads below have more than 32 targets (several
32-test tiles per gene), empty columns, and genes that do not fit in shared memory.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_p_close, gene_major_to_target_major

pytestmark = pytest.mark.gpu

ZH = {"none": 0, "min": 1, "max": 2, "mix": 3}
ALT = {"less": 0, "greater": 1, "two-sided": 2}


def _with_empty_columns(w, every=7):
    """Drops the entries of every `every`-th column (the column stays, with no entries)."""
    keep = np.ones(w.indices.size, bool)
    counts = np.diff(w.indptr)
    for c in range(0, w.n_cols, every):
        keep[w.indptr[c]:w.indptr[c + 1]] = False
        counts[c] = 0
    w.data = w.data[keep]
    w.indices = w.indices[keep]
    w.indptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return w


def _fused_separate(w, **opt):
    from hpdex_gb300.resident import ResidentMatrix, BATCHED, PLAIN
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    plan = M.plan(w.group_id, w.n_targets, **opt)
    plan.run(BATCHED)
    fused = plan.download()
    plan.run(PLAIN)
    fused_plain = plan.download()
    plan.set_fused_pvalues(False)
    plan.run(BATCHED)
    separate = plan.download()
    plan.set_fused_pvalues(True)
    plan.run(BATCHED)  # the graph is captured again with the fused stage
    again = plan.download()
    for U1, P in (fused_plain, separate, again):
        np.testing.assert_array_equal(U1, fused[0])
        np.testing.assert_array_equal(P, fused[1])
    return fused


@pytest.mark.parametrize("zh", ["min", "max", "mix"])
@pytest.mark.parametrize("alt", ["two-sided", "less", "greater"])
def test_fused_equals_separate_and_oracle(zh, alt):
    from oracle import oracle
    from hpdex_gb300 import synthetic
    w = _with_empty_columns(synthetic.perturb_screen(seed=13, n_rows=12_000, n_cols=150,
                                                     n_targets=70, ref_size=1_500))
    U1, P = _fused_separate(w, zero_handling=zh, alternative=alt, use_continuity=True,
                            fast_norm=False)
    U1o, Po = oracle.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                  tie_correction=True, use_continuity=True,
                                  zero_handling=ZH[zh], alternative=ALT[alt], method=2, threads=-1)
    C, T = w.n_cols, w.n_targets
    np.testing.assert_array_equal(U1, gene_major_to_target_major(U1o, C, T))
    assert_p_close(P, gene_major_to_target_major(Po, C, T))


@pytest.mark.parametrize("alt", ["two-sided", "less", "greater"])
def test_fused_none_mode_and_fast_norm(alt):
    """zero_handling none (n1, n2 per gene and test) and the fast normal tail, fused."""
    from hpdex_gb300 import synthetic
    w = synthetic.exact_small(seed=8, n_rows=3_000, n_cols=64, n_targets=40, ref_size=200)
    w.data = np.round(w.data * 8) / 8
    _fused_separate(w, zero_handling="none", alternative=alt, use_continuity=False,
                    fast_norm=False)
    _fused_separate(w, zero_handling="none", alternative=alt, use_continuity=True,
                    fast_norm=True)
    u = synthetic.umi_counts(seed=3, n_rows=6_000, n_cols=120, n_targets=45)
    _fused_separate(u, zero_handling="mix", alternative=alt, use_continuity=True, fast_norm=True)


def test_fused_large_columns():
    """Genes longer than the shared-memory capacity (several slabs; the pending tests are
    taken in the first slab's rank phase), with a tie-free and a tie-heavy column mix."""
    from hpdex_gb300 import synthetic
    w = synthetic.umi_counts(seed=17, n_rows=120_000, n_cols=40, n_targets=36)
    _fused_separate(w, zero_handling="min", use_continuity=True, fast_norm=False)
    w.data = w.data + np.random.default_rng(1).random(w.data.size).astype(w.data.dtype)
    _fused_separate(w, zero_handling="max", use_continuity=False, fast_norm=False)


def test_fused_oversized_buckets_and_many_groups():
    """Columns above the shared-memory capacity with one dominant value (a bucket of more
    than 65,535 elements, ranked in place in global memory) and packed distinct keys; then
    2,000 targets (accumulators in shared memory, run counters in global memory) and 7,000
    targets (accumulators in global memory too, 32-bit group ids). The fused plan equals the
    one-shot call (separate p-value kernel) bit for bit."""
    from test_gpu_large_columns import COLUMNS, _workload
    from hpdex_gb300.backend.bin import kernel
    rng = np.random.default_rng(2)
    cases = [_workload(3, 150_000, COLUMNS, 30_000,
                       [500, 800, 1200, 2000, 3000, 4500, 6000, 700, 650, 5200, 900, 3300]),
             _workload(5, 60_000, COLUMNS[:3], 8_000, list(rng.integers(20, 26, size=2_000))),
             _workload(6, 45_000, COLUMNS[:3], 6_000, list(rng.integers(3, 7, size=7_000)))]
    from test_gpu_parity import _oracle_compare
    assert _oracle_compare(cases[-1], zero_handling="min") == "ok"
    for w in cases:
        U1, P = _fused_separate(w, zero_handling="min", use_continuity=True, fast_norm=False)
        U1o, Po = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                      use_continuity=True, zero_handling=1, fast_norm=False)
        np.testing.assert_array_equal(U1, U1o)
        np.testing.assert_array_equal(P, Po)
