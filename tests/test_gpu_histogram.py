"""GPU: the rank kernel's histogram path (genes whose stored values are small integers, as UMI
counts are) against its bucket path and the oracle.

A gene takes the histogram path when every stored finite value is an integer of magnitude
below 2^31 and its value span times the number of groups fits the kernel's shared memory;
other genes of the same launch take the bucket path. Bars: U1 and P of the histogram path equal
the bucket path's bit for bit (resident plans with the path switched on and off), and the
oracle's (U1 bit-exact, P within 1e-12 relative, absolute floor 1e-300), over every integer
dtype and float data holding integers, negative values, the four zero modes, the three
alternatives, value spans too wide for the counters (per-gene fallback), non-integral and
out-of-range values (bucket path), and the duplicate-row-id error.
"""
from types import SimpleNamespace

import numpy as np
import pytest

from test_gpu_parity import _oracle_compare

pytestmark = pytest.mark.gpu

ZH = {"none": 0, "min": 1, "max": 2, "mix": 3}


def _integer_workload(seed, dtype, n_rows=6_000, n_cols=80, n_targets=12, signed=False,
                      spread=40, dense=False, wide_every=0, nonint_col=None):
    """CSC of integer counts (NB-like via geometric draws), optionally signed; every
    `wide_every`-th gene gets a value span of about 20,000 (too many counters for the
    histogram); column `nonint_col` holds one non-integral value."""
    rng = np.random.default_rng(seed)
    data, indices, indptr = [], [], [0]
    for j in range(n_cols):
        dens = 1.0 if dense else float(rng.uniform(0.05, 0.9))
        rows = np.nonzero(rng.random(n_rows) < dens)[0]
        v = rng.geometric(1.0 / (1.0 + rng.uniform(0.5, spread)), rows.size).astype(np.int64)
        if signed:
            v *= rng.choice(np.array([-1, 1]), rows.size)
        if wide_every and j % wide_every == 0:
            v[: max(1, rows.size // 50)] = 20_000
        x = v.astype(dtype)
        if nonint_col is not None and j == nonint_col and x.size:
            x = x.astype(np.float64) if np.dtype(dtype).kind != "f" else x
            x[0] = 2.5
            x = x.astype(dtype)
        data.append(x)
        indices.append(rows.astype(np.int64))
        indptr.append(indptr[-1] + rows.size)
    gid = np.full(n_rows, -1, np.int32)
    perm = rng.permutation(n_rows)
    ref = n_rows // 4
    gid[perm[:ref]] = 0
    rest = perm[ref: int(0.97 * n_rows)]
    gid[rest] = rng.integers(1, n_targets + 1, rest.size).astype(np.int32)
    return SimpleNamespace(data=np.concatenate(data), indices=np.concatenate(indices),
                           indptr=np.asarray(indptr, np.int64), n_rows=n_rows, n_cols=n_cols,
                           n_targets=n_targets, group_id=gid)


def _both_paths(w, **opt):
    from hpdex_gb300.resident import BATCHED, ResidentMatrix
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    try:
        plan = M.plan(w.group_id, w.n_targets, **opt)
        plan.run(BATCHED)
        U1h, Ph = plan.download()
        plan.set_histogram(False)
        plan.run(BATCHED)
        U1b, Pb = plan.download()
        plan.close()
    finally:
        M.close()
    return (U1h, Ph), (U1b, Pb)


@pytest.mark.parametrize("dtype", [np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32,
                                   np.int64, np.uint64, np.float32, np.float64])
def test_histogram_equals_bucket_path_and_oracle(dtype):
    signed = np.dtype(dtype).kind in "if"
    w = _integer_workload(int(np.dtype(dtype).num), dtype, signed=signed,
                          spread=20 if np.dtype(dtype).itemsize == 1 else 60)
    for zh in ("min", "mix") if signed else ("min", "max"):
        (U1h, Ph), (U1b, Pb) = _both_paths(w, zero_handling=zh, use_continuity=True)
        np.testing.assert_array_equal(U1h, U1b)
        np.testing.assert_array_equal(Ph, Pb)
        assert _oracle_compare(w, zero_handling=zh) == "ok"


@pytest.mark.parametrize("alt", [0, 1, 2])
def test_histogram_none_mode_all_alternatives(alt):
    """zero_handling='none' ranks explicit zeros too: dense signed counts with zeros."""
    w = _integer_workload(77 + alt, np.int16, n_rows=3_000, n_cols=50, signed=True, dense=True,
                          spread=6)
    w.data[::7] = 0
    (U1h, Ph), (U1b, Pb) = _both_paths(w, zero_handling="none", alternative=alt,
                                       tie_correction=bool(alt != 1))
    np.testing.assert_array_equal(U1h, U1b)
    np.testing.assert_array_equal(Ph, Pb)
    assert _oracle_compare(w, zero_handling="none", alternative=alt,
                           tie_correction=bool(alt != 1)) == "ok"


def test_histogram_mixed_with_bucket_genes():
    """Wide value spans, a non-integral value and many targets send some genes of the launch to
    the bucket path: both kinds in one launch, the same results."""
    w = _integer_workload(5, np.float32, n_rows=20_000, n_cols=120, n_targets=300, wide_every=7,
                          nonint_col=3)
    (U1h, Ph), (U1b, Pb) = _both_paths(w, zero_handling="min", use_continuity=True)
    np.testing.assert_array_equal(U1h, U1b)
    np.testing.assert_array_equal(Ph, Pb)
    assert _oracle_compare(w, zero_handling="min") == "ok"


def test_histogram_out_of_range_integers_take_the_bucket_path():
    """Integers at or above 2^31 in magnitude (uint32 and int64) are not counted in bins."""
    for dtype, big in ((np.uint32, 2**31 + 5), (np.int64, -(2**31) - 3), (np.int64, 2**40)):
        w = _integer_workload(9, dtype, n_rows=4_000, n_cols=30)
        w.data[::97] = big
        (U1h, Ph), (U1b, Pb) = _both_paths(w, zero_handling="min")
        np.testing.assert_array_equal(U1h, U1b)
        np.testing.assert_array_equal(Ph, Pb)
        assert _oracle_compare(w, zero_handling="min") == "ok"


def test_umi_counts_histogram_path_matches_oracle():
    from hpdex_gb300 import synthetic
    w = synthetic.umi_counts(seed=6, n_rows=20_000, n_cols=300, n_targets=49)
    (U1h, Ph), (U1b, Pb) = _both_paths(w, zero_handling="min", use_continuity=True)
    np.testing.assert_array_equal(U1h, U1b)
    np.testing.assert_array_equal(Ph, Pb)
    assert _oracle_compare(w, zero_handling="min") == "ok"


def test_histogram_duplicate_row_ids_raise():
    """A column storing more entries for a group than the group has rows (duplicate row ids)
    raises the same error on both paths."""
    from hpdex_gb300.backend.bin import kernel
    rng = np.random.default_rng(2)
    n_rows = 200
    gid = np.zeros(n_rows, np.int32)
    gid[100:] = 1
    rows = np.concatenate([np.arange(n_rows), np.arange(100, 200)])  # group 1 stored twice
    data = rng.integers(1, 5, rows.size).astype(np.float32)
    indptr = np.array([0, rows.size], np.int64)
    with pytest.raises(RuntimeError, match="duplicate row indices"):
        kernel.mannwhitneyu(data, rows, indptr, gid, 1, zero_handling=1, fast_norm=False)
