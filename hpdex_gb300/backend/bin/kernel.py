"""Drop-in for the reference's compiled module `hpdex.backend.bin.kernel`.

Same functions, argument names, defaults and error behaviour as the reference binding
(AI4Cell/hpdex src/cpp/module.cpp:193-243, typed in src/hpdex/backend/kernel.pyi), backed
by the GB300 library through its C ABI (include/hpdex_gb300.h). Differences, by design:
  * mannwhitneyu returns U1 and P as read-only float64 arrays of shape
    (n_targets, n_genes); the reference returns flat gene-major arrays, so
    reference_U1.reshape(n_genes, n_targets).T equals U1 here.
  * layout="csr" means the arrays describe a genes x cells CSR matrix (the wrapper's
    contract, mannwhitneyu_.py:51-58), which is the same memory as a cells x genes CSC; the
    reference's binding swaps the row/column counts for CSR instead (module.cpp:51-58).
  * fast_norm=True (the binding's default, as in the reference) selects the reference's fast
    normal tail, its scalar form (Numerical Recipes erfcc, ~1e-7 relative); the reference's
    vectorised form nests the polynomial differently, so its fast values are not reproduced
    bit for bit. The wrapper hpdex_gb300.backend.mannwhitneyu defaults to fast_norm=False.
  * threads only affects host-side preparation.
  * indices may be int32 (scipy's index type): they are passed to the device as they are,
    without the cast to int64 that the reference's wrapper does; any other integer type is
    cast to int64 as before. The results are the same.
  * U1 and P live in page-locked buffers from the library's pool when one is available (the
    device writes them directly); a buffer returns to the pool with its array.
"""
from __future__ import annotations

import sys
import time

import numpy as np

from ... import _lib

__all__ = ["mannwhitneyu", "group_mean"]

_DTYPES = {np.dtype(k): v for k, v in _lib.DTYPE_CODES.items()}


def _as_data(data):
    data = np.asarray(data)
    if data.dtype not in _DTYPES:
        raise RuntimeError("Unsupported dtype for data")
    return np.ascontiguousarray(data)


def _as_index(a):
    return np.ascontiguousarray(np.asarray(a), dtype=np.int64)


def _check_size(name, v):
    v = int(v)
    if v < 0:
        raise TypeError(f"{name} must be a non-negative integer")
    return v


def _readonly(a):
    a.flags.writeable = False
    return a


def _options(ref_sorted, tar_sorted, tie_correction, use_continuity, fast_norm, zero_handling,
             alternative, method, exact_variant=0):
    o = _lib.MwuOptions()
    o.ref_sorted = int(bool(ref_sorted))
    o.tar_sorted = int(bool(tar_sorted))
    o.tie_correction = int(bool(tie_correction))
    o.use_continuity = int(bool(use_continuity))
    o.fast_norm = int(bool(fast_norm))
    o.zero_handling = int(zero_handling)
    o.alternative = int(alternative)
    o.method = int(method)
    o.exact_variant = int(exact_variant)
    return o


def mannwhitneyu(data, indices, indptr, group_id, n_targets, ref_sorted=False, tar_sorted=False,
                 tie_correction=True, use_continuity=False, fast_norm=True, zero_handling=0,
                 alternative=2, method=2, threads=-1, layout="csc", show_progress=False,
                 exact_variant=0):
    """Mann-Whitney U per (gene, target) of a CSC matrix grouped by `group_id`.

    `exact_variant` (extension, method=1 only): 0 reproduces the reference's exact p-values,
    1 uses the true MWU null distribution (scipy semantics). int32 `indices` are taken as they
    are (extension).
    Returns (U1, P), each float64 of shape (n_targets, n_genes), read-only."""
    n_targets = _check_size("n_targets", n_targets)
    data = _as_data(data)
    indices = np.asarray(indices)
    # int32 row ids (scipy's index type) go to the device as they are: half the bytes to
    # upload and no host cast; anything else is cast to int64 as the reference binding takes
    idx32 = indices.dtype == np.int32
    indices = np.ascontiguousarray(indices) if idx32 else _as_index(indices)
    indptr = _as_index(indptr)
    group_id = np.ascontiguousarray(np.asarray(group_id), dtype=np.int32)
    R, C, nnz = group_id.size, indptr.size - 1, data.size
    if C < 0:
        raise RuntimeError("indptr must have at least one entry")
    if indices.size < nnz:
        raise RuntimeError("indices is shorter than data")
    opt = _options(ref_sorted, tar_sorted, tie_correction, use_continuity, fast_norm,
                   zero_handling, alternative, method, exact_variant)
    U1 = _lib.result_array((max(n_targets, 0), C))
    P = _lib.result_array((max(n_targets, 0), C))
    t0 = time.perf_counter()
    entry = _lib.lib().hpdex_mannwhitneyu_idx32 if idx32 else _lib.lib().hpdex_mannwhitneyu
    st = entry(_DTYPES[data.dtype], data.ctypes.data, indices.ctypes.data, indptr.ctypes.data, R, C,
               nnz, group_id.ctypes.data, n_targets, opt, int(threads), U1.ctypes.data,
               P.ctypes.data)
    _lib.check(st)
    if show_progress:
        print(f"[hpdex_gb300] mannwhitneyu: {C} genes x {n_targets} targets in "
              f"{time.perf_counter() - t0:.4f} s", file=sys.stderr)
    return _readonly(U1), _readonly(P)


def group_mean(data, indices, indptr, group_id, n_groups, include_zeros=True, threads=-1,
               use_kahan=False, layout="csc"):
    """Per (gene, group) means, flat [gene * n_groups + g] (the reference's layout)."""
    n_groups = _check_size("n_groups", n_groups)
    data = _as_data(data)
    indices = _as_index(indices)
    indptr = _as_index(indptr)
    group_id = np.ascontiguousarray(np.asarray(group_id), dtype=np.int32)
    R, C, nnz = group_id.size, indptr.size - 1, data.size
    out = np.zeros(max(C, 0) * n_groups, np.float64)
    if n_groups == 0 or C <= 0:
        return _readonly(out)
    st = _lib.lib().hpdex_group_mean(_DTYPES[data.dtype], data.ctypes.data, indices.ctypes.data,
                                     indptr.ctypes.data, R, C, nnz, group_id.ctypes.data,
                                     n_groups, int(bool(include_zeros)), int(bool(use_kahan)),
                                     int(threads), out.ctypes.data)
    _lib.check(st)
    return _readonly(out)
