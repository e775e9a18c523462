"""The seeded synthetic workloads that stand in for the benchmark configurations: shapes,
densities, group layouts and value properties as the hot-path specification states them (with
its recorded resolutions), checked at reduced column counts so that the CPU suite stays fast."""
import numpy as np

from hpdex_gb300 import synthetic


def _valid_csc(w):
    assert w.indptr[0] == 0 and w.indptr[-1] == w.data.size == w.indices.size
    assert np.all(np.diff(w.indptr) >= 0)
    for c in range(0, w.n_cols, max(1, w.n_cols // 50)):
        r = w.indices[w.indptr[c]:w.indptr[c + 1]]
        assert np.all(np.diff(r) > 0) and (r.size == 0 or (r[0] >= 0 and r[-1] < w.n_rows))
    assert w.group_id.size == w.n_rows and w.group_id.dtype == np.int32


def test_perturb_screen_shape_density_and_groups():
    w = synthetic.perturb_screen(n_cols=600)
    _valid_csc(w)
    assert (w.n_rows, w.n_targets) == (200_000, 500)
    density = w.data.size / (w.n_rows * w.n_cols)
    assert 0.07 < density < 0.11  # gene density ~ Beta(0.5, 5): about 9 %
    assert w.data.dtype == np.float32 and np.all(np.isfinite(w.data)) and np.all(w.data > 0)
    g = w.group_id
    assert np.sum(g == 0) == 20_000
    sizes = np.bincount(g[g > 0], minlength=w.n_targets + 1)[1:]
    assert sizes.size == 500 and sizes.min() >= 20 and sizes.max() <= 3000
    assert 20_000 + sizes.sum() <= w.n_rows  # scaled to fit the 180,000 other cells
    assert np.all((g >= -1) & (g <= w.n_targets))


def test_perturb_screen_values_are_log1p_cp10k():
    """Stored values are log1p(count / library size * 1e4): per cell, expm1 of its values sums
    to 1e4 (CP10k)."""
    w = synthetic.perturb_screen(n_cols=400, seed=3)
    per_cell = np.bincount(w.indices, weights=np.expm1(w.data.astype(np.float64)), minlength=w.n_rows)
    stored = np.bincount(w.indices, minlength=w.n_rows) > 0
    np.testing.assert_allclose(per_cell[stored], 1e4, rtol=1e-4)


def test_umi_counts_realised_density_and_groups():
    w = synthetic.umi_counts(n_cols=300)
    _valid_csc(w)
    assert np.all(w.data == np.round(w.data)) and np.all(w.data >= 1)  # integral counts
    density = w.data.size / (w.n_rows * w.n_cols)
    assert 0.25 < density < 0.45  # NB size 2: ~35 % realised (not the nominal 7 %)
    g = w.group_id
    assert np.sum(g == 0) == 10_000
    assert np.sum(g >= 0) <= int(0.98 * w.n_rows) + w.n_targets  # ~98 % assigned, rest -1


def test_exact_small_is_dense_with_small_groups():
    w = synthetic.exact_small(n_cols=50, n_targets=200)
    _valid_csc(w)
    assert w.data.size == w.n_rows * w.n_cols  # dense, stored as CSC
    g = w.group_id
    assert np.sum(g == 0) == 40
    sizes = np.bincount(g[g > 0], minlength=w.n_targets + 1)[1:]
    assert sizes.min() >= 3 and sizes.max() <= 40  # at most 38 distinct (n1, n2) pairs


def test_umi_counts_low_location_variant_hits_the_nominal_density():
    """With the mean's log-location at -3.5 instead of -1 the same NB model gives the nominal
    ~7 % density."""
    w = synthetic.umi_counts(n_cols=400, mu_log_loc=-3.5)
    _valid_csc(w)
    density = w.data.size / (w.n_rows * w.n_cols)
    assert 0.05 < density < 0.09
