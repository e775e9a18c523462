"""The no-allocation entry point against the regular one, through the C ABI.

hpdex_mannwhitneyu_noalloc serves callers that must not allocate device memory during a
call (framework memory pools, pre-reserved serving loops, plugin hosts): they hand in
device buffers and the library works inside one fixed scratch array. This test builds
those device buffers with torch (test plumbing only), calls the entry point twice in a row
on different inputs -- the second call finds the first call's leftovers in the shared
scratch -- and requires the same U1 and P as hpdex_mannwhitneyu on the same host arrays.
U1 must be bit-exact and P within 1e-12 relative (absolute floor 1e-300), the tolerance
of the other parity tests. This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _regular(w, opt):
    from hpdex_gb300.backend.bin import kernel
    return kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                               tie_correction=bool(opt.tie_correction),
                               use_continuity=bool(opt.use_continuity),
                               zero_handling=opt.zero_handling, alternative=opt.alternative,
                               fast_norm=bool(opt.fast_norm))


def _noalloc(w, opt, torch):
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
    _lib.check(st)
    torch.cuda.synchronize()
    return U1.cpu().numpy(), P.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch sees no CUDA device")
    from hpdex_gb300 import synthetic
    from hpdex_gb300.resident import make_options
    cases = [
        (synthetic.perturb_screen(seed=31, n_rows=30_000, n_cols=400, n_targets=80, ref_size=3_000),
         make_options(tie_correction=True, use_continuity=True, zero_handling="min")),
        (synthetic.umi_counts(seed=12, n_rows=12_000, n_cols=250, n_targets=20),
         make_options(tie_correction=True, use_continuity=False, zero_handling="mix",
                      alternative="greater")),
    ]
    for w, opt in cases:  # two calls in a row on the shared scratch
        U1r, Pr = _regular(w, opt)
        U1n, Pn = _noalloc(w, opt, torch)
        np.testing.assert_array_equal(U1n, U1r)
        bad = np.abs(Pn - Pr) > np.maximum(1e-12 * np.abs(Pr), 1e-300)
        assert not bad.any(), np.max(np.abs(Pn - Pr) / np.maximum(Pr, 1e-300))
