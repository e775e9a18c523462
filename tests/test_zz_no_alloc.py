"""The no-allocation entry point against the regular one, through the C ABI.

hpdex_mannwhitneyu_noalloc serves callers that must not allocate device memory during a
call (framework memory pools, pre-reserved serving loops, plugin hosts): they hand in
device buffers and the library works inside one fixed scratch array. This test builds
those device buffers with torch (test plumbing only), calls the entry point several times in
a row on different inputs -- each call finds the previous call's leftovers in the shared
scratch -- and requires the same U1 and P as hpdex_mannwhitneyu on the same host arrays.
U1 must be bit-exact and P within 1e-12 relative (absolute floor 1e-300), the tolerance
of the other parity tests. The cases cover zero_handling none / min / mix, a column longer
than the rank kernel's shared-memory capacity (its slabs go through the second scratch slice),
and the limits, which must come back as HPDEX_ERR_UNSUPPORTED with a message. This file is
named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from hpdex_gb300.synthetic import Workload

pytestmark = pytest.mark.gpu


def _regular(w, opt):
    from hpdex_gb300.backend.bin import kernel
    return kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                               tie_correction=bool(opt.tie_correction),
                               use_continuity=bool(opt.use_continuity),
                               zero_handling=opt.zero_handling, alternative=opt.alternative,
                               fast_norm=bool(opt.fast_norm))


def _call(w, opt, torch):
    """(status, message, U1, P) of one no-allocation call on device copies of w."""
    from hpdex_gb300 import _lib
    dev = torch.device("cuda:0")
    data = torch.from_numpy(np.ascontiguousarray(w.data)).to(dev)
    rows = torch.from_numpy(w.indices.astype(np.int32)).to(dev)
    indptr = torch.from_numpy(w.indptr.astype(np.int64)).to(dev)
    gid = torch.from_numpy(w.group_id.astype(np.int32)).to(dev)
    U1 = torch.empty((w.n_targets, w.n_cols), dtype=torch.float64, device=dev)
    P = torch.empty((w.n_targets, w.n_cols), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    st = _lib.lib().hpdex_mannwhitneyu_noalloc(
        _lib.DTYPE_CODES[w.data.dtype.name], data.data_ptr(), rows.data_ptr(), indptr.data_ptr(),
        w.n_rows, w.n_cols, gid.data_ptr(), w.n_targets, ctypes.byref(opt), U1.data_ptr(),
        P.data_ptr(), None)
    msg = _lib.lib().hpdex_last_error().decode() if st else ""
    torch.cuda.synchronize()
    return st, msg, U1.cpu().numpy(), P.cpu().numpy()


def _noalloc(w, opt, torch):
    from hpdex_gb300 import _lib
    st, msg, U1, P = _call(w, opt, torch)
    if st:
        raise _lib.HpdexError(st, msg)
    return U1, P


def _long_column_case(seed=3, n_rows=40_000):
    """Three genes: one with about 30,000 stored entries (above the rank kernel's shared-memory
    element capacity, so its slabs are scattered into the second per-CTA scratch slice), two
    sparse ones; 20,000 reference cells and 4 targets."""
    rng = np.random.default_rng(seed)
    cols = []
    for dens in (0.75, 0.05, 0.3):
        rows = np.nonzero(rng.random(n_rows) < dens)[0]
        vals = np.round(rng.gamma(2.0, 1.5, rows.size) * 4.0) / 4.0 + 0.25
        cols.append((rows, vals.astype(np.float32)))
    indptr = np.cumsum([0] + [r.size for r, _ in cols]).astype(np.int64)
    gid = np.zeros(n_rows, np.int32)
    gid[rng.permutation(n_rows)[: n_rows // 2]] = rng.integers(1, 5, n_rows // 2).astype(np.int32)
    return Workload("long_column", n_rows, 3, np.concatenate([v for _, v in cols]),
                    np.concatenate([r for r, _ in cols]).astype(np.int64), indptr, gid, 4, {})


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("torch sees no CUDA device")
    return t


def test_noalloc_matches_regular_entry_point_in_a_row(torch):
    from hpdex_gb300 import synthetic
    from hpdex_gb300.resident import make_options
    long_col = _long_column_case()
    assert np.diff(long_col.indptr).max() > 25_000
    cases = [
        (synthetic.perturb_screen(seed=31, n_rows=30_000, n_cols=400, n_targets=80, ref_size=3_000),
         make_options(tie_correction=True, use_continuity=True, zero_handling="min")),
        (synthetic.umi_counts(seed=12, n_rows=12_000, n_cols=250, n_targets=20),
         make_options(tie_correction=True, use_continuity=False, zero_handling="mix",
                      alternative="greater")),
        (synthetic.umi_counts(seed=13, n_rows=6_000, n_cols=60, n_targets=5, mu_log_loc=2.5),
         make_options(tie_correction=True, use_continuity=True, zero_handling="none")),
        (long_col, make_options(tie_correction=True, use_continuity=True, zero_handling="min")),
        (long_col, make_options(tie_correction=False, use_continuity=False, zero_handling="max",
                                alternative="less")),
    ]
    for w, opt in cases:  # calls in a row on the shared scratch
        U1r, Pr = _regular(w, opt)
        U1n, Pn = _noalloc(w, opt, torch)
        np.testing.assert_array_equal(U1n, U1r)
        bad = np.abs(Pn - Pr) > np.maximum(1e-12 * np.abs(Pr), 1e-300)
        assert not bad.any(), np.max(np.abs(Pn - Pr) / np.maximum(Pr, 1e-300))


def test_noalloc_limits_are_reported(torch):
    from hpdex_gb300 import _lib
    from hpdex_gb300.resident import make_options
    opt = make_options(tie_correction=True, use_continuity=True, zero_handling="min")
    rng = np.random.default_rng(5)
    # too many groups: n_targets + 1 above HPDEX_NOALLOC_MAX_GROUPS (1024)
    n_rows = 4_000
    w = Workload("many_groups", n_rows, 2, rng.random(200).astype(np.float32),
                 np.sort(rng.choice(n_rows, 200, replace=False)).astype(np.int64) % n_rows,
                 np.array([0, 100, 200], np.int64), (np.arange(n_rows) % 1025).astype(np.int32),
                 1024, {})
    st, msg, _, _ = _call(w, opt, torch)
    assert st == _lib.HPDEX_ERR_UNSUPPORTED and "exceeds 1024" in msg, (st, msg)
    # a column longer than the scratch slices allow (a dense 120,000-cell column)
    n_rows = 120_000
    w = Workload("dense_column", n_rows, 1, rng.random(n_rows).astype(np.float32),
                 np.arange(n_rows, dtype=np.int64), np.array([0, n_rows], np.int64),
                 (np.arange(n_rows) % 3).astype(np.int32), 2, {})
    st, msg, _, _ = _call(w, opt, torch)
    assert st == _lib.HPDEX_ERR_UNSUPPORTED and "column holds 120000 entries" in msg, (st, msg)
    # exact p-values are not offered here
    st, msg, _, _ = _call(w, make_options(method="exact"), torch)
    assert st == _lib.HPDEX_ERR_UNSUPPORTED and "asymptotic only" in msg, (st, msg)
    # the shared scratch is still usable after the refusals
    w = _long_column_case(seed=4)
    U1r, Pr = _regular(w, opt)
    U1n, Pn = _noalloc(w, opt, torch)
    np.testing.assert_array_equal(U1n, U1r)
    assert np.all(np.abs(Pn - Pr) <= np.maximum(1e-12 * np.abs(Pr), 1e-300))
