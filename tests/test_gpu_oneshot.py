"""GPU: the pipelined one-shot call (column chunks uploaded while earlier chunks are ranked,
p-values written straight into the output arrays on coherent-memory systems) returns what the
resident path returns, also after the device memory cache is released, and across dtypes."""
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _resident(w, **opt):
    from hpdex_gb300.resident import ResidentMatrix
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    plan = M.plan(w.group_id, w.n_targets, **opt)
    plan.run()
    return plan.download()


@pytest.mark.parametrize("zh,zname", [(1, "min"), (2, "max"), (3, "mix")])
def test_oneshot_equals_resident(zh, zname):
    from hpdex_gb300 import synthetic
    from hpdex_gb300.backend.bin import kernel
    w = synthetic.perturb_screen(seed=31, n_rows=30_000, n_cols=700, n_targets=40, ref_size=3_000)
    U1r, Pr = _resident(w, zero_handling=zname, use_continuity=True)
    for _ in range(2):  # second call reuses cached device memory
        U1, P = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                    use_continuity=True, zero_handling=zh, fast_norm=False)
        np.testing.assert_array_equal(U1, U1r)
        np.testing.assert_array_equal(P, Pr)


def test_release_cached_memory_between_calls():
    import hpdex_gb300
    from hpdex_gb300 import synthetic
    from hpdex_gb300.backend.bin import kernel
    w = synthetic.umi_counts(seed=6, n_rows=6_000, n_cols=150, n_targets=9)
    a = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets, zero_handling=1, fast_norm=False)
    hpdex_gb300.release_cached_memory()
    b = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets, zero_handling=1, fast_norm=False)
    hpdex_gb300.release_cached_memory()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("dtype", [np.int16, np.uint32, np.float64, np.int64])
def test_oneshot_dtypes_equal_resident(dtype):
    from hpdex_gb300 import synthetic
    from hpdex_gb300.backend.bin import kernel
    w = synthetic.umi_counts(seed=12, n_rows=8_000, n_cols=160, n_targets=12)
    w.data = w.data.astype(dtype)
    U1r, Pr = _resident(w, zero_handling="min", use_continuity=False)
    U1, P = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                zero_handling=1, fast_norm=False)
    np.testing.assert_array_equal(U1, U1r)
    np.testing.assert_array_equal(P, Pr)


def test_results_in_pooled_page_locked_buffers():
    """The wrapper's result arrays come from the library's page-locked buffer pool: released
    with the arrays, reused by the next call, never shared with a result still alive."""
    import hpdex_gb300
    from hpdex_gb300 import synthetic
    from hpdex_gb300.backend.bin import kernel
    w = synthetic.umi_counts(seed=6, n_rows=6_000, n_cols=150, n_targets=9)
    hpdex_gb300.release_cached_memory()  # no idle buffers left over from earlier tests
    call = lambda: kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                       zero_handling=1, fast_norm=False)
    a = call()
    assert type(a[0].base.base).__name__ == "PinnedBuffer"
    addr = {a[0].ctypes.data, a[1].ctypes.data}
    ref = (a[0].copy(), a[1].copy())
    del a
    b = call()
    assert {b[0].ctypes.data, b[1].ctypes.data} == addr  # the released buffers were reused
    c = call()  # b is alive: c gets other buffers, and b keeps its values
    assert not ({c[0].ctypes.data, c[1].ctypes.data} & addr)
    for U1, P in (b, c):
        np.testing.assert_array_equal(U1, ref[0])
        np.testing.assert_array_equal(P, ref[1])


@pytest.mark.parametrize("zh", [0, 1, 3])
def test_int32_row_ids_equal_int64(zh):
    """Row ids given as int32 (uploaded as they are) give the int64 path's results, also with
    row ids outside [0, n_rows), which both skip as the reference does."""
    from hpdex_gb300 import synthetic
    from hpdex_gb300.backend.bin import kernel
    w = synthetic.exact_small(seed=8, n_rows=3_000, n_cols=64, n_targets=40, ref_size=200)
    w.data = np.round(w.data * 8) / 8
    idx64 = w.indices.astype(np.int64).copy()
    idx64[::97] = w.n_rows + 5
    idx64[13::89] = -3
    idx32 = idx64.astype(np.int32)
    kw = dict(use_continuity=True, zero_handling=zh, fast_norm=False)
    try:
        r64 = kernel.mannwhitneyu(w.data, idx64, w.indptr, w.group_id, w.n_targets, **kw)
    except RuntimeError as e:
        with pytest.raises(RuntimeError, match=re.escape(str(e))):
            kernel.mannwhitneyu(w.data, idx32, w.indptr, w.group_id, w.n_targets, **kw)
        return
    r32 = kernel.mannwhitneyu(w.data, idx32, w.indptr, w.group_id, w.n_targets, **kw)
    np.testing.assert_array_equal(r32[0], r64[0])
    np.testing.assert_array_equal(r32[1], r64[1])


def test_int32_row_ids_resident_matrix():
    """A resident matrix built from int32 row ids (with ids outside [0, n_rows)) gives the
    int64-built matrix's results and group means."""
    from hpdex_gb300 import synthetic
    from hpdex_gb300.resident import ResidentMatrix
    w = synthetic.umi_counts(seed=5, n_rows=8_000, n_cols=120, n_targets=12)
    idx64 = w.indices.astype(np.int64).copy()
    idx64[::101] = w.n_rows + 7
    idx64[7::103] = -1
    out = []
    for idx in (idx64, idx64.astype(np.int32)):
        M = ResidentMatrix(w.data, idx, w.indptr, w.n_rows)
        plan = M.plan(w.group_id, w.n_targets, zero_handling="min", use_continuity=True)
        plan.run()
        out.append((*plan.download(), M.group_mean(w.group_id, w.n_targets + 1)))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.float32, np.float64])
def test_upload_at_every_alignment(dtype):
    """The one-shot call reads the caller's arrays in 16-byte words from the first entry of a
    chunk where host and device arrays are all aligned, element by element before it, after
    the last whole quad, and everywhere when the host arrays cannot be aligned. Value and row-id
    arrays placed 0-5 elements into larger buffers (int64 and int32 row ids, ids outside
    [0, n_rows) among them) give the resident path's results bit for bit."""
    from hpdex_gb300 import synthetic
    from hpdex_gb300.backend.bin import kernel
    w = synthetic.umi_counts(seed=21, n_rows=9_000, n_cols=137, n_targets=11)
    w.data = w.data.astype(dtype)
    idx = w.indices.astype(np.int64).copy()
    idx[::89] = w.n_rows + 3
    idx[5::97] = -2
    w.indices = idx
    U1r, Pr = _resident(w, zero_handling="min", use_continuity=True)
    nnz = w.data.size

    def placed(a, off):
        buf = np.zeros(a.size + 8, a.dtype)
        v = buf[off:off + a.size]
        v[:] = a
        return v

    for off_v, off_r in ((0, 0), (1, 0), (0, 1), (2, 3), (4, 2), (5, 5)):
        for rows in (idx, idx.astype(np.int32)):
            U1, P = kernel.mannwhitneyu(placed(w.data, off_v), placed(rows, off_r), w.indptr,
                                        w.group_id, w.n_targets, use_continuity=True,
                                        zero_handling=1, fast_norm=False)
            np.testing.assert_array_equal(U1, U1r)
            np.testing.assert_array_equal(P, Pr)
    assert nnz > 12 * 4


def test_pageable_output_arrays():
    """Outputs in ordinary (pageable, never written) numpy arrays: on coherent-memory systems the
    p-value kernels of both compute streams write them directly, after a host thread has touched
    their pages; elsewhere the results are copied back. Either way the results equal the
    wrapper's (page-locked outputs), on a workload of several chunks."""
    import ctypes
    from hpdex_gb300 import _lib, synthetic
    from hpdex_gb300.backend.bin import kernel
    from hpdex_gb300.resident import make_options
    w = synthetic.perturb_screen(seed=33, n_rows=40_000, n_cols=900, n_targets=60, ref_size=4_000)
    U1r, Pr = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                  use_continuity=True, zero_handling=1, fast_norm=False)
    opt = make_options(tie_correction=True, use_continuity=True, zero_handling="min")
    for _ in range(2):
        U1 = np.empty((w.n_targets, w.n_cols))
        P = np.empty((w.n_targets, w.n_cols))
        st = _lib.lib().hpdex_mannwhitneyu(
            _lib.DTYPE_CODES[w.data.dtype.name], w.data.ctypes.data, w.indices.ctypes.data,
            w.indptr.ctypes.data, w.n_rows, w.n_cols, w.data.size, w.group_id.ctypes.data,
            w.n_targets, ctypes.byref(opt), -1, U1.ctypes.data, P.ctypes.data)
        assert st == 0, _lib.lib().hpdex_last_error()
        np.testing.assert_array_equal(U1, U1r)
        np.testing.assert_array_equal(P, Pr)
