"""Exact-mode p-values on the GPU, at the exact configuration's sizes.

Workload: dense N(0, 1) float32 with a per-(target, gene) shift, 60,000 cells x 4,000 genes
stored as CSC (2.4e8 values), a reference of 40 cells and 1,500 targets of 3-40 cells, so at
most 38 distinct (n1, n2) tables. Two variants are checked:

- exact_variant=0 reproduces the reference's exact p. The reference's DP counts compositions
  in wrapping uint64, and at n1 = 40 it wraps. Every 10th gene is compared with the oracle:
  U1 bit-exact, P within 1e-12 relative (absolute floor 1e-300).
- exact_variant=1 uses the true MWU null, built as double counts on the device. It is compared
  with the exact-integer null (oracle/exact_null.py): every test of small workloads, and 20,000
  sampled tests of the full one, within 1e-12 relative. A numpy restatement of the device's
  double DP stays within 3e-15 of the exact null at n1 = 40, n2 = 3..40.

Size-independent properties are checked on every test of the full run: 2 U1 integral,
0 <= U1 <= n1 n2, P in [0, 1].
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P_RTOL = 1e-12
P_FLOOR = 1e-300


def assert_p_close(P, Pref):
    P, Pref = np.asarray(P), np.asarray(Pref)
    bad = np.abs(P - Pref) > np.maximum(P_RTOL * np.abs(Pref), P_FLOOR)
    if bad.any():
        err = np.abs(P - Pref) / np.maximum(np.abs(Pref), P_FLOOR)
        raise AssertionError(f"{int(bad.sum())} p-values off, max rel err {err.max():.3e}")


def sizes_of(w):
    """n1 and n2 per target. The data are dense, so every zero mode counts every cell."""
    g = w.group_id
    s = np.bincount(g[(g >= 0) & (g <= w.n_targets)], minlength=w.n_targets + 1)
    return int(s[0]), s[1:].astype(np.int64)


def columns(w, sel):
    sizes = np.diff(w.indptr)[sel]
    ip = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    idx = np.concatenate([np.arange(w.indptr[c], w.indptr[c + 1]) for c in sel])
    return w.data[idx], w.indices[idx], ip


def gpu_exact(w, data, indices, indptr, zh, alt, variant):
    from hpdex_gb300.backend.bin import kernel
    return kernel.mannwhitneyu(data, indices, indptr, w.group_id, w.n_targets,
                               tie_correction=True, use_continuity=False, zero_handling=zh,
                               alternative=alt, method=1, exact_variant=variant,
                               fast_norm=False)


def null_p(U1, n1, n2, alt):
    from oracle.exact_null import p_exact
    return np.array([p_exact(float(u), n1, int(b), alt) for u, b in zip(U1, n2)])


@pytest.fixture(scope="module")
def exact_screen():
    from hpdex_gb300 import synthetic
    w = synthetic.exact_small()
    assert (w.n_rows, w.n_cols, w.n_targets, w.nnz) == (60_000, 4_000, 1_500, 240_000_000)
    return w


@pytest.mark.parametrize("alt", [0, 1, 2])
@pytest.mark.parametrize("zh", [0, 1])
def test_true_null_every_test_of_small_workloads(zh, alt):
    from hpdex_gb300 import synthetic
    w = synthetic.exact_small(seed=19, n_rows=3_000, n_cols=24, n_targets=40)
    n1, n2 = sizes_of(w)
    U1, P = gpu_exact(w, w.data, w.indices, w.indptr, zh, alt, 1)
    for t in range(w.n_targets):
        assert_p_close(P[t], null_p(U1[t], n1, np.full(w.n_cols, n2[t]), alt))


def test_reference_variant_full_size(exact_screen):
    from oracle import oracle
    w = exact_screen
    U1, P = gpu_exact(w, w.data, w.indices, w.indptr, 0, 2, 0)
    n1, n2 = sizes_of(w)
    assert np.all(2.0 * U1 == np.round(2.0 * U1))
    assert np.all((U1 >= 0) & (U1 <= (n1 * n2)[:, None]))
    assert np.all((P >= 0.0) & (P <= 1.0))
    sel = np.arange(0, w.n_cols, 10)
    d, i, ip = columns(w, sel)
    U1o, Po = oracle.mannwhitneyu(d, i, ip, w.group_id, w.n_targets, tie_correction=True,
                                  use_continuity=False, zero_handling=0, alternative=2,
                                  method=1, threads=-1)
    np.testing.assert_array_equal(U1[:, sel], U1o.reshape(sel.size, w.n_targets).T)
    assert_p_close(P[:, sel], Po.reshape(sel.size, w.n_targets).T)


def test_true_null_full_size(exact_screen):
    w = exact_screen
    U1, P = gpu_exact(w, w.data, w.indices, w.indptr, 1, 2, 1)
    n1, n2 = sizes_of(w)
    assert np.all((P >= 0.0) & (P <= 1.0))
    rng = np.random.default_rng(3)
    t = rng.integers(0, w.n_targets, size=20_000)
    c = rng.integers(0, w.n_cols, size=20_000)
    assert_p_close(P[t, c], null_p(U1[t, c], n1, n2[t], 2))
