"""ctypes binding of the native library libhpdex_gb300.so (C ABI in include/hpdex_gb300.h).

The library is the only compute path: there is no CPU fallback. Loading fails loudly when
the library has not been built, and every call raises when no CUDA device is usable.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

_lock = threading.Lock()
_lib = None

DTYPE_CODES = {
    "int8": 0, "uint8": 1, "int16": 2, "uint16": 3, "int32": 4, "uint32": 5,
    "int64": 6, "uint64": 7, "float32": 8, "float64": 9,
}

(HPDEX_OK, HPDEX_ERR_RUNTIME, HPDEX_ERR_ARGUMENT, HPDEX_ERR_CUDA, HPDEX_ERR_UNSUPPORTED,
 HPDEX_ERR_TIMEOUT) = range(6)


class MwuOptions(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "ref_sorted", "tar_sorted", "tie_correction", "use_continuity", "fast_norm",
        "zero_handling", "alternative", "method", "exact_variant")]


class HpdexError(RuntimeError):
    """Raised for every non-OK status; reference-style runtime errors keep their text."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


EXPORTS = {
    # name: (restype, argtypes)
    "hpdex_mwu_options_default": (None, [ctypes.POINTER(MwuOptions)]),
    "hpdex_last_error": (ctypes.c_char_p, []),
    "hpdex_device_count": (ctypes.c_int, []),
    "hpdex_device_sm_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32)]),
    "hpdex_release_cached_memory": (ctypes.c_int, []),
    "hpdex_host_buffer_acquire": (ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "hpdex_host_buffer_release": (ctypes.c_int, [ctypes.c_void_p]),
    "hpdex_selftest_erfc": (ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double)]),
    "hpdex_selftest_erfc_values": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "hpdex_selftest_division": (ctypes.c_int, [ctypes.c_int64, ctypes.c_uint64,
                                               ctypes.POINTER(ctypes.c_int64)]),
    "hpdex_bh_fdr": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "hpdex_fold_change": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "hpdex_mannwhitneyu": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                          ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.POINTER(MwuOptions), ctypes.c_int32,
                                          ctypes.c_void_p, ctypes.c_void_p]),
    "hpdex_mannwhitneyu_idx32": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                                ctypes.POINTER(MwuOptions), ctypes.c_int32,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "hpdex_group_mean": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_void_p]),
    "hpdex_matrix_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                           ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "hpdex_matrix_create_idx32": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                           ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "hpdex_matrix_create_device": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                  ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "hpdex_matrix_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "hpdex_matrix_create_csr": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                               ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "hpdex_matrix_create_csr_idx32": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                               ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "hpdex_matrix_group_mean": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                               ctypes.c_int32, ctypes.c_void_p]),
    "hpdex_matrix_info": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int64)] * 4),
    "hpdex_plan_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                         ctypes.POINTER(MwuOptions),
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "hpdex_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "hpdex_plan_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "hpdex_plan_download": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "hpdex_plan_set_fused_pvalues": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "hpdex_plan_set_drain_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "hpdex_plan_set_run_counters": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "hpdex_plan_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p]),
    "hpdex_plan_set_histogram": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "hpdex_plan_set_bucket_bits": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "hpdex_plan_timings": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float),
                                          ctypes.POINTER(ctypes.c_int32)]),
    "hpdex_mannwhitneyu_noalloc": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                  ctypes.c_void_p, ctypes.c_int64,
                                                  ctypes.POINTER(MwuOptions), ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p]),
    "hpdex_server_create": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int32,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "hpdex_server_add_matrix": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.POINTER(ctypes.c_int32)]),
    "hpdex_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.POINTER(MwuOptions),
                                           ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_int64)]),
    "hpdex_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
                                         ctypes.POINTER(ctypes.c_double)]),
    "hpdex_server_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.POINTER(ctypes.c_int64),
                                          ctypes.POINTER(ctypes.c_double)]),
    "hpdex_server_phase_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_double)]),
    "hpdex_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
}


def lib_path() -> str:
    return _build.LIB


def lib():
    """Loads libhpdex_gb300.so (building it first when the sources are newer)."""
    global _lib
    with _lock:
        if _lib is None:
            if not _build.up_to_date():
                try:
                    _build.build()
                except Exception as e:  # no nvcc: fail loudly, never fall back
                    if not os.path.exists(_build.LIB):
                        raise RuntimeError(f"hpdex_gb300 native library is missing and could not be built: {e}")
            L = ctypes.CDLL(_build.LIB)
            for name, (res, args) in EXPORTS.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(status: int) -> None:
    if status != HPDEX_OK:
        msg = lib().hpdex_last_error().decode(errors="replace")
        raise HpdexError(status, msg)


def device_count() -> int:
    return int(lib().hpdex_device_count())


def release_cached_memory() -> None:
    """Return the device memory (and idle page-locked result buffers) that finished calls keep
    cached for reuse to the driver."""
    check(lib().hpdex_release_cached_memory())


_PINNED_TYPES = {}


def _pinned_release(self):
    try:
        lib().hpdex_host_buffer_release(ctypes.addressof(self))
    except Exception:  # interpreter shutdown
        pass


def result_array(shape):
    """A float64 array for results: backed by a page-locked buffer from the library's pool when
    one is available (the device then writes it directly; the buffer goes back to the pool
    when the array and its views are gone), else ordinary memory."""
    import numpy as np
    n = 1
    for d in shape:
        n *= int(d)
    nbytes = 8 * n
    if nbytes == 0:
        return np.empty(shape, np.float64)
    ptr = ctypes.c_void_p()
    if lib().hpdex_host_buffer_acquire(nbytes, ctypes.byref(ptr)) != 0 or not ptr.value:
        return np.empty(shape, np.float64)
    T = _PINNED_TYPES.get(nbytes)
    if T is None:
        T = type("PinnedBuffer", (ctypes.c_char * nbytes,), {"__del__": _pinned_release})
        _PINNED_TYPES[nbytes] = T
    buf = T.from_address(ptr.value)
    return np.frombuffer(buf, dtype=np.float64, count=n).reshape(shape)


def bh_fdr(p):
    """Benjamini-Hochberg adjusted p-values on the device (scipy's false_discovery_control)."""
    import numpy as np
    p = np.ascontiguousarray(np.asarray(p, dtype=np.float64)).reshape(-1)
    out = np.empty_like(p)
    check(lib().hpdex_bh_fdr(p.ctypes.data, p.size, out.ctypes.data))
    return out


def fold_change(means_gene_major, n_genes: int, n_groups: int, clip_value: float):
    """(fold, log2 fold), each (n_groups - 1, n_genes), from gene-major group means."""
    import numpy as np
    m = np.ascontiguousarray(np.asarray(means_gene_major, dtype=np.float64)).reshape(-1)
    if m.size != n_genes * n_groups:
        raise ValueError("means must hold n_genes * n_groups values")
    fold = np.empty((max(n_groups - 1, 0), n_genes), np.float64)
    log2fold = np.empty_like(fold)
    check(lib().hpdex_fold_change(m.ctypes.data, int(n_genes), int(n_groups), float(clip_value),
                                  fold.ctypes.data, log2fold.ctypes.data))
    return fold, log2fold
