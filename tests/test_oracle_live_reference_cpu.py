"""The oracle against the reference's own compiled kernel, live, on fresh seeded inputs.

tests/golden/ pins the oracle to 61 stored outputs of the reference. Where the reference's
kernel has been built here (oracle/build_ref.sh compiles src/cpp/module.cpp and
mannwhitneyu.cpp, unmodified, into oracle/_ref/), this file adds a randomised sweep run
against that kernel directly: 240 cases over the ten value dtypes, the four zero modes, the
three alternatives, continuity and tie correction on and off, asymptotic and exact p-values,
explicit zeros, NaN/+-Inf, out-of-range and negative row ids, rows in no group and groups
too small to test. The oracle must return the same U1 and P bit for bit, or the same error
text, and the same group means in both summation modes.

The reference is called with fast_norm=False (its fast path needs Highway, absent here; the
scalar fast path is pinned in tests/test_fast_norm_pin_cpu.py). Its binding forwards
`threads` into `use_kahan` (module.cpp:211-213), so threads=0 gives the plain sum and
threads=1 the Kahan sum.
"""
import glob
import importlib.util
import os

import numpy as np
import pytest

from conftest import ROOT

DTYPES = [np.float32, np.float64, np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32,
          np.int64, np.uint64]


@pytest.fixture(scope="module")
def ref_kernel():
    found = glob.glob(os.path.join(ROOT, "oracle", "_ref", "kernel*.so"))
    if not found:
        pytest.skip("the reference's kernel was not built here (sources absent)")
    spec = importlib.util.spec_from_file_location("kernel", found[0])
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _case(rng, k):
    dtype = DTYPES[k % len(DTYPES)]
    exact = k % 6 == 5
    R = int(rng.integers(20, 50)) if exact else int(rng.integers(30, 400))
    C = int(rng.integers(1, 10))
    T = int(rng.integers(1, 6))
    zh = int(rng.integers(0, 4))
    X = rng.standard_normal((R, C))
    if k % 3:
        X = np.round(X * 2.0)                      # ties
    if k % 2:
        X = np.abs(X)
    dens = rng.uniform(0.8, 1.0) if zh == 0 else rng.uniform(0.05, 0.95)
    X[rng.random((R, C)) > dens] = 0.0
    if np.issubdtype(dtype, np.integer):
        X = np.round(X * 3.0)
        if np.issubdtype(dtype, np.unsignedinteger):
            X = np.abs(X)
        info = np.iinfo(dtype)
        X = np.clip(X, info.min, info.max)
    X = X.astype(dtype)
    if k % 4 == 0 and np.issubdtype(dtype, np.floating):
        X[rng.random((R, C)) < 0.05] = np.nan
        X[rng.random((R, C)) < 0.03] = np.inf
        X[rng.random((R, C)) < 0.03] = -np.inf
    if k % 8 == 0:
        X[rng.random((R, C)) < 0.1] = 0               # some explicitly stored zeros below
    stored = (X != 0) | ~np.isfinite(X.astype(np.float64))
    if k % 8 == 0:
        stored |= rng.random((R, C)) < 0.1
    cols, rows = np.nonzero(stored.T)               # column-major: CSC order
    data = X[rows, cols]
    indptr = np.searchsorted(cols, np.arange(C + 1)).astype(np.int64)
    indices = rows.astype(np.int64)
    if k % 5 == 0 and indices.size > 4:
        j = rng.choice(indices.size, size=2, replace=False)
        indices[j[0]], indices[j[1]] = R + 3, -2    # skipped by the reference
    gid = rng.integers(-1, T + 2, R).astype(np.int32)
    gid[: 2 * (T + 1)] = np.repeat(np.arange(T + 1), 2)
    if k % 7 == 0:                                  # one group left with a single row
        g0 = k % (T + 1)
        rows_g0 = np.nonzero(gid == g0)[0]
        gid[rows_g0[1:]] = -1
    o = dict(tie_correction=bool(k % 2), use_continuity=bool((k // 2) % 2), zero_handling=zh,
             alternative=int(rng.integers(0, 3)), method=1 if exact else 2)
    return data, indices, indptr, gid, T, o


@pytest.mark.parametrize("block", range(8))
def test_oracle_equals_reference_kernel_on_random_cases(ref_kernel, oracle_lib, block):
    rng = np.random.default_rng(1000 + block)
    for k in range(block * 30, block * 30 + 30):
        data, indices, indptr, gid, T, o = _case(rng, k)
        try:
            U1r, Pr = ref_kernel.mannwhitneyu(data, indices, indptr, gid, T, False, False,
                                              o["tie_correction"], o["use_continuity"], False,
                                              o["zero_handling"], o["alternative"], o["method"],
                                              1, "csc", False)
            err_r = ""
        except RuntimeError as e:
            err_r = str(e)
        try:
            U1o, Po = oracle_lib.mannwhitneyu(data, indices, indptr, gid, T, threads=2, **o)
            err_o = ""
        except RuntimeError as e:
            err_o = str(e)
        assert err_o == err_r, (k, o)
        if not err_r:
            np.testing.assert_array_equal(U1o, np.asarray(U1r), err_msg=f"case {k} {o}")
            np.testing.assert_array_equal(Po, np.asarray(Pr), err_msg=f"case {k} {o}")
        for include_zeros in (True, False):
            for kahan in (False, True):
                mr = ref_kernel.group_mean(data, indices, indptr, gid, T + 1, include_zeros,
                                           int(kahan), False, "csc")
                mo = oracle_lib.group_mean(data, indices, indptr, gid, T + 1, include_zeros, 2,
                                           kahan)
                np.testing.assert_array_equal(mo, np.asarray(mr), err_msg=f"means {k}")


@pytest.mark.parametrize("alt", [0, 1, 2])
def test_oracle_exact_reference_variant_at_forty_reference_cells(ref_kernel, oracle_lib, alt):
    """The exact configuration's shape: 40 reference cells and targets of 3-40 cells, where the
    reference's uint64 composition count wraps. The oracle must wrap the same way."""
    from hpdex_gb300 import synthetic
    w = synthetic.exact_small(seed=23, n_rows=4_000, n_cols=5, n_targets=60, ref_size=40)
    args = (w.data, w.indices, w.indptr, w.group_id, w.n_targets)
    U1r, Pr = ref_kernel.mannwhitneyu(*args, False, False, True, False, False, 0, alt, 1, 1,
                                      "csc", False)
    U1o, Po = oracle_lib.mannwhitneyu(*args, tie_correction=True, use_continuity=False,
                                      zero_handling=0, alternative=alt, method=1, threads=2)
    np.testing.assert_array_equal(U1o, np.asarray(U1r))
    np.testing.assert_array_equal(Po, np.asarray(Pr))
    sizes = np.bincount(w.group_id[w.group_id >= 0], minlength=w.n_targets + 1)
    assert sizes[0] == 40 and sizes[1:].max() >= 30


@pytest.mark.parametrize("zh", [1, 2, 3])
@pytest.mark.parametrize("workload", ["perturb_screen", "umi_counts"])
def test_oracle_equals_reference_kernel_on_scaled_workloads(ref_kernel, oracle_lib, workload, zh):
    """Scaled-down copies of the benchmark's screen and of the integer-count workload
    (heavy ties), in the zero modes that place an implicit-zero block."""
    from hpdex_gb300 import synthetic
    if workload == "perturb_screen":
        w = synthetic.perturb_screen(seed=101, n_rows=30_000, n_cols=300, n_targets=60,
                                     ref_size=3_000)
    else:
        w = synthetic.umi_counts(seed=102, n_rows=20_000, n_cols=200, n_targets=20)
    args = (w.data, w.indices.astype(np.int64), w.indptr, w.group_id, w.n_targets)
    U1r, Pr = ref_kernel.mannwhitneyu(*args, False, False, True, True, False, zh, 2, 2, 1,
                                      "csc", False)
    U1o, Po = oracle_lib.mannwhitneyu(*args, tie_correction=True, use_continuity=True,
                                      zero_handling=zh, alternative=2, method=2, threads=-1)
    np.testing.assert_array_equal(U1o, np.asarray(U1r))
    np.testing.assert_array_equal(Po, np.asarray(Pr))
