"""GPU: cells x genes CSR input (AnnData's native layout) transposed on the device. The
resident matrix it builds gives the same tests and group means as the host-built CSC, also
with gene ids outside the matrix (dropped), empty rows and columns, and more genes than the
shared-memory cursor table holds; the DE driver gives the same table for CSR and CSC input."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def _groups(n, rng, ref=300, T=6):
    gid = np.full(n, -1, np.int32)
    perm = rng.permutation(n)
    gid[perm[:ref]] = 0
    o = ref
    for t in range(1, T + 1):
        s = int(rng.integers(40, 200))
        gid[perm[o:o + s]] = t
        o += s
    return gid, T


def _compare(Xcsr, gid, T):
    from hpdex_gb300.resident import ResidentMatrix
    Xcsc = Xcsr.tocsc()
    Mr = ResidentMatrix.from_scipy(Xcsr)  # int32 gene ids, uploaded as they are
    Mr64 = ResidentMatrix.from_csr(Xcsr.data, Xcsr.indices.astype(np.int64), Xcsr.indptr,
                                   *Xcsr.shape)
    Mc = ResidentMatrix(Xcsc.data, Xcsc.indices, Xcsc.indptr, Xcsc.shape[0])
    Mc64 = ResidentMatrix(Xcsc.data, Xcsc.indices.astype(np.int64), Xcsc.indptr, Xcsc.shape[0])
    assert Mr.nnz == Mr64.nnz == Xcsc.nnz
    out = []
    for M in (Mr, Mc, Mr64, Mc64):
        p = M.plan(gid, T, zero_handling="min", use_continuity=True)
        p.run()
        out.append(p.download() + (M.group_mean(gid, T + 1),))
    for other in out[1:]:
        for a, b in zip(out[0], other):
            np.testing.assert_array_equal(a, b)


def test_csr_random_float():
    rng = np.random.default_rng(1)
    X = sp.random(3_000, 900, density=0.08, format="csr", random_state=2, dtype=np.float32)
    X.data = np.round(X.data * 20).astype(np.float32) / 4  # ties
    X = sp.csr_matrix(X)
    X[5] = 0  # an empty row
    X.eliminate_zeros()
    gid, T = _groups(X.shape[0], rng)
    _compare(X, gid, T)


def test_csr_many_genes_global_cursors():
    rng = np.random.default_rng(3)
    X = sp.random(1_500, 60_000, density=0.004, format="csr", random_state=4, dtype=np.float64)
    gid, T = _groups(X.shape[0], rng, ref=200, T=3)
    _compare(X, gid, T)


def test_csr_out_of_range_gene_ids_are_dropped():
    from hpdex_gb300.resident import ResidentMatrix
    rng = np.random.default_rng(5)
    X = sp.random(800, 300, density=0.1, format="csr", random_state=6, dtype=np.float32)
    indices = X.indices.astype(np.int64).copy()
    bad = rng.random(indices.size) < 0.05
    indices[bad] = np.where(rng.random(bad.sum()) < 0.5, -1, 300 + 7)
    keep = ~bad
    rows = np.repeat(np.arange(X.shape[0]), np.diff(X.indptr))
    good = sp.csc_matrix((X.data[keep], (rows[keep], indices[keep])), shape=X.shape)
    good.sort_indices()
    gid, T = _groups(X.shape[0], rng, ref=150, T=3)
    Mr = ResidentMatrix.from_csr(X.data, indices, X.indptr, X.shape[0], X.shape[1])
    Mr32 = ResidentMatrix.from_csr(X.data, indices.astype(np.int32), X.indptr, X.shape[0], X.shape[1])
    Mc = ResidentMatrix(good.data, good.indices, good.indptr, good.shape[0])
    assert Mr.nnz == Mr32.nnz == good.nnz
    res = []
    for M in (Mr, Mc, Mr32):
        p = M.plan(gid, T, zero_handling="mix")
        p.run()
        res.append(p.download())
    for other in res[1:]:
        np.testing.assert_array_equal(res[0][0], other[0])
        np.testing.assert_array_equal(res[0][1], other[1])


def test_de_driver_csr_equals_csc():
    from hpdex_gb300 import differential_expression, synthetic
    w = synthetic.umi_counts(seed=10, n_rows=5_000, n_cols=140, n_targets=5)
    Xc = sp.csc_matrix((w.data, w.indices, w.indptr), shape=(w.n_rows, w.n_cols))
    labels = np.where(w.group_id == 0, "ref", np.char.add("t", w.group_id.astype(str)))
    a = differential_expression(Xc, labels, "ref")
    b = differential_expression(Xc.tocsr(), labels, "ref")
    for k in a:
        if a[k].dtype == object:
            assert list(a[k]) == list(b[k])
        else:
            np.testing.assert_array_equal(a[k], b[k])
