"""Host-side logic that needs no GPU: the wrappers' argument checks and option maps (as in
the reference's src/hpdex/backend/mannwhitneyu_.py) and the DE driver's group selection
(src/hpdex/de.py:57-87)."""
import numpy as np
import pytest
import scipy.sparse as sp

from hpdex_gb300.backend import mannwhitneyu_ as W
from hpdex_gb300 import de


def test_wrapper_rejects_dense_and_bad_group_id():
    X = np.ones((4, 3), np.float32)
    with pytest.raises(ValueError, match="CSR or CSC"):
        W.mannwhitneyu(X, np.zeros(4, np.int32), 1)
    with pytest.raises(ValueError, match="length 4"):
        W.mannwhitneyu(sp.csc_matrix(X), np.zeros(3, np.int32), 1)
    # CSR: group_id runs over the columns (genes x cells contract)
    with pytest.raises(ValueError, match="length 3"):
        W.group_mean(sp.csr_matrix(X), np.zeros(4, np.int32), 2)


def test_option_maps_match_reference():
    assert W._zero_handling_map == {"none": 0, "min": 1, "max": 2, "mix": 3}
    assert W._alternative_map == {"less": 0, "greater": 1, "two-sided": 2}
    assert W._method_map == {"exact": 1, "asymptotic": 2}


def test_sparse_parts_casts_like_reference():
    X = sp.csc_matrix(np.eye(5, dtype=np.float64))
    X.indices = X.indices.astype(np.int64)
    data, ind, ptr, gid, layout = W._sparse_parts(X, np.arange(5, dtype=np.int64))
    assert ind.dtype == np.int64 and ptr.dtype == np.int64 and gid.dtype == np.int32
    assert layout == "csc"
    # int32 row ids (scipy's default) are passed on as int32, without a host cast
    Y = sp.csc_matrix(np.eye(5, dtype=np.float64))
    assert Y.indices.dtype == np.int32
    _, ind32, ptr32, _, _ = W._sparse_parts(Y, np.arange(5))
    assert ind32.dtype == np.int32 and ptr32.dtype == np.int64


def test_de_group_selection():
    labels = np.array(["ctl", "a", "b", "a", "ctl", "c", "b"], dtype=object)
    assert de._select_groups(labels, "ctl", None, 2) == ["a", "b"]   # c has 1 sample
    assert de._select_groups(labels, "ctl", ["b", "zz", "ctl"], 1) == ["b"]
    with pytest.raises(ValueError, match="Reference"):
        de._select_groups(labels, "nope", None, 1)
    with pytest.raises(ValueError, match="No valid target groups"):
        de._select_groups(np.array(["ctl", "ctl"], dtype=object), "ctl", None, 1)
