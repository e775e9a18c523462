"""GPU: the DE driver's post-processing on the device. BH FDR equals
scipy.stats.false_discovery_control(method="bh") bit for bit (ties, zeros, ones, several
radix-sort tile boundaries, 4 million values); out-of-range input raises scipy's message;
fold change / log2 fold change equal the reference driver's numpy expressions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 3, 10, 2047, 2048, 2049, 100_003, 4_000_000])
def test_bh_equals_scipy(n):
    from scipy.stats import false_discovery_control
    from hpdex_gb300._lib import bh_fdr
    rng = np.random.default_rng(n)
    p = rng.random(n) ** 3
    tie = rng.random(n) < 0.3
    p[tie] = rng.choice(p[: min(7, n)], size=int(tie.sum()))
    p[rng.random(n) < 0.02] = 0.0
    p[rng.random(n) < 0.02] = 1.0
    p[rng.random(n) < 0.01] = 1e-300
    ref = false_discovery_control(p, method="bh") if n > 1 else p.copy()
    np.testing.assert_array_equal(bh_fdr(p), ref)


def test_bh_rejects_values_outside_unit_interval():
    from hpdex_gb300._lib import bh_fdr
    for bad in (np.array([0.1, 1.5, 0.2]), np.array([0.1, np.nan, 0.3]), np.array([-0.1, 0.5])):
        with pytest.raises(RuntimeError, match="must lie between 0. and 1."):
            bh_fdr(bad)


def test_fold_change_equals_reference_expressions():
    from hpdex_gb300._lib import fold_change
    rng = np.random.default_rng(3)
    n_genes, G, clip = 5_000, 7, 20.0
    means = rng.gamma(0.5, 2.0, size=(n_genes, G))
    means[rng.random((n_genes, G)) < 0.1] = 0.0
    means[rng.random((n_genes, G)) < 0.05] = 1e-12
    fold, log2fold = fold_change(means.reshape(-1), n_genes, G, clip)
    m = means.T
    ref_means, tar_means = m[0], m[1:]
    with np.errstate(divide="ignore", invalid="ignore"):
        f = tar_means / ref_means
        f = np.where(ref_means < 1e-10, clip, f)
        f = np.where(tar_means < 1e-10, 1.0 / clip, f)
        l2 = np.log2(f)
    np.testing.assert_array_equal(fold, f)
    np.testing.assert_allclose(log2fold, l2, rtol=1e-12, atol=0)


def test_de_driver_fdr_matches_scipy():
    from scipy.stats import false_discovery_control
    from hpdex_gb300 import differential_expression, synthetic
    import scipy.sparse as sp
    w = synthetic.umi_counts(seed=8, n_rows=6_000, n_cols=120, n_targets=6)
    X = sp.csc_matrix((w.data, w.indices, w.indptr), shape=(w.n_rows, w.n_cols))
    labels = np.where(w.group_id < 0, "ignored", np.char.add("g", w.group_id.astype(str)))
    labels = np.where(w.group_id == 0, "ref", labels)
    out = differential_expression(X, labels, "ref")
    np.testing.assert_array_equal(out["fdr"], false_discovery_control(out["p_value"], method="bh"))
