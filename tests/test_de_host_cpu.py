"""The DE driver's host logic on the CPU (hpdex_gb300/de.py against the reference's
src/hpdex/de.py:35-198).

differential_expression does its arithmetic on the device (group means, fold change, the
tests, BH). Here those calls are replaced by CPU stand-ins -- the oracle for the means and
the tests, the reference driver's own numpy fold change (de.py:138-142) and scipy's BH
(de.py:174-184) -- so that what remains is the driver itself: group selection, the group-id
map, the flattening and the row labels. The device calls are covered by the GPU tests
(tests/test_gpu_de_post.py). Checks:
- the seven columns of the reference schema, in its order;
- row t * n_genes + j carries target groups[t] and feature j, and its p_value / u_statistic
  are the oracle's for that (target, gene) pair (the reference pairs them wrongly when there
  is more than one target; the rebuild keeps labels and values together);
- fold_change and log2_fold_change follow the reference formula from the group means
  computed independently (dense numpy, zeros included);
- fdr is scipy's BH of the p_value column;
- CSR, CSC and dense inputs give the same table, and groups below min_samples are dropped.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from hpdex_gb300 import _lib, de, resident


def false_discovery_control(p, method="bh"):
    from scipy.stats import false_discovery_control as fdc  # scipy >= 1.11
    return fdc(p, method=method)


CLIP = 20.0


class _Plan:
    def __init__(self, X, group_id, n_targets, opts):
        self.X, self.gid, self.T, self.opts = X, group_id, n_targets, opts

    def run(self):
        pass

    def download(self):
        from oracle import oracle
        X = self.X
        U1, P = oracle.mannwhitneyu(X.data, X.indices, X.indptr, self.gid, self.T,
                                    tie_correction=self.opts["tie_correction"],
                                    use_continuity=self.opts["use_continuity"],
                                    zero_handling=resident._ZH[self.opts["zero_handling"]],
                                    alternative=2, method=2, threads=1)
        C = X.shape[1]
        return U1.reshape(C, self.T).T, P.reshape(C, self.T).T


class _Resident:
    @classmethod
    def from_scipy(cls, X):
        self = cls()
        self.X = sp.csc_matrix(X)
        return self

    def group_mean(self, group_id, n_groups, include_zeros=True):
        from oracle import oracle
        X = self.X
        return oracle.group_mean(X.data, X.indices, X.indptr, group_id, n_groups,
                                 include_zeros=include_zeros, threads=1)

    def plan(self, group_id, n_targets, **opts):
        return _Plan(self.X, np.asarray(group_id, np.int32), n_targets, opts)


def _fold_change_reference(means_gene_major, n_genes, n_groups, clip_value):
    means = np.asarray(means_gene_major).reshape(n_genes, n_groups).T
    ref, tar = means[0], means[1:]
    with np.errstate(divide="ignore", invalid="ignore"):
        fc = tar / ref
        fc = np.where(ref < 1e-10, clip_value, fc)
        fc = np.where(tar < 1e-10, 1.0 / clip_value, fc)
        return fc, np.log2(fc)


@pytest.fixture
def cpu_device(monkeypatch):
    monkeypatch.setattr(resident, "ResidentMatrix", _Resident)
    monkeypatch.setattr(_lib, "fold_change", _fold_change_reference)
    monkeypatch.setattr(_lib, "bh_fdr", lambda p: false_discovery_control(p, method="bh"))


def _dataset(seed=5, n_cells=600, n_genes=40):
    rng = np.random.default_rng(seed)
    dens = rng.uniform(0.05, 0.6, size=n_genes)
    X = np.where(rng.random((n_cells, n_genes)) < dens,
                 np.log1p(rng.poisson(3.0, (n_cells, n_genes)) + 1.0), 0.0).astype(np.float32)
    X[:, 7] = 0.0  # a gene with no stored values: fold change hits both clips
    labels = rng.choice(np.array(["ctl", "kd1", "kd2", "kd3", "rare"], dtype=object),
                        size=n_cells, p=[0.4, 0.2, 0.2, 0.195, 0.005])
    labels[:3] = "rare"
    labels[3:] = np.where(labels[3:] == "rare", "ctl", labels[3:])  # exactly 3 "rare" cells
    features = np.array([f"g{j}" for j in range(n_genes)], dtype=object)
    return X, labels, features


def test_table_pairs_labels_with_their_values(cpu_device):
    from oracle import oracle
    X, labels, features = _dataset()
    out = de.differential_expression(sp.csc_matrix(X), labels, "ctl", features=features,
                                     min_samples=4, clip_value=CLIP)
    assert list(out) == de.COLUMNS
    groups = [g for g in dict.fromkeys(labels.tolist()) if g not in ("ctl", "rare")]
    T, C = len(groups), X.shape[1]
    assert all(v.shape == (T * C,) for v in out.values())
    # independent group ids and statistics, test by test
    gid = np.full(labels.size, -1, np.int32)
    gid[labels == "ctl"] = 0
    Xc = sp.csc_matrix(X)
    for t, g in enumerate(groups):
        gid_t = np.where(labels == g, 1, np.where(labels == "ctl", 0, -1)).astype(np.int32)
        U1, P = oracle.mannwhitneyu(Xc.data, Xc.indices, Xc.indptr, gid_t, 1,
                                    tie_correction=True, use_continuity=True, zero_handling=1,
                                    alternative=2, method=2, threads=1)
        rows = slice(t * C, (t + 1) * C)
        assert np.all(out["target"][rows] == g)
        assert np.all(out["feature"][rows] == features)
        np.testing.assert_array_equal(out["u_statistic"][rows], U1)
        np.testing.assert_array_equal(out["p_value"][rows], P)
        ref_mean = X[labels == "ctl"].astype(np.float64).mean(axis=0)
        tar_mean = X[labels == g].astype(np.float64).mean(axis=0)
        with np.errstate(divide="ignore", invalid="ignore"):
            fc = np.where(tar_mean < 1e-10, 1.0 / CLIP,
                          np.where(ref_mean < 1e-10, CLIP, tar_mean / ref_mean))
        np.testing.assert_allclose(out["fold_change"][rows], fc, rtol=1e-6)
        np.testing.assert_allclose(out["log2_fold_change"][rows], np.log2(fc), rtol=1e-6,
                                   atol=1e-9)
    assert out["fold_change"][7] == 1.0 / CLIP  # empty gene: the target clip wins
    np.testing.assert_array_equal(out["fdr"], false_discovery_control(out["p_value"], method="bh"))


def test_layouts_give_the_same_table_and_small_groups_are_dropped(cpu_device):
    X, labels, features = _dataset(seed=9)
    a = de.differential_expression(sp.csc_matrix(X), labels, "ctl", min_samples=4)
    b = de.differential_expression(sp.csr_matrix(X), labels, "ctl", min_samples=4)
    c = de.differential_expression(X, labels, "ctl", min_samples=4)
    for k in de.COLUMNS:
        np.testing.assert_array_equal(a[k], b[k])
        np.testing.assert_array_equal(a[k], c[k])
    assert "rare" not in set(a["target"])
    d = de.differential_expression(X, labels, "ctl", min_samples=2)
    assert "rare" in set(d["target"])
    assert np.array_equal(a["feature"][:X.shape[1]], np.arange(X.shape[1]).astype(object))


def test_unsupported_metric_and_missing_reference(cpu_device):
    X, labels, _ = _dataset()
    with pytest.raises(ValueError, match="Unsupported metric"):
        de.differential_expression(X, labels, "ctl", metric="t-test")
    with pytest.raises(ValueError, match="Reference"):
        de.differential_expression(X, labels, "nope")
