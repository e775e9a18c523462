"""ctypes front-end of the CPU oracle (oracle/mwu_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
legs. The hpdex_gb300 package never imports this module.

`mannwhitneyu` / `group_mean` take the same raw CSC arrays and integer options as the
reference binding `kernel.mannwhitneyu` / `kernel.group_mean`
(AI4Cell/hpdex src/cpp/module.cpp:193-243) and return gene-major flat arrays exactly as
the reference does (src/cpp/mannwhitneyu.cpp:959), raising RuntimeError with the
reference's messages.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

DTYPE_CODES = {
    np.dtype(np.int8): 0, np.dtype(np.uint8): 1, np.dtype(np.int16): 2, np.dtype(np.uint16): 3,
    np.dtype(np.int32): 4, np.dtype(np.uint32): 5, np.dtype(np.int64): 6, np.dtype(np.uint64): 7,
    np.dtype(np.float32): 8, np.dtype(np.float64): 9,
}


def build() -> str:
    """Compiles liboracle.so with the committed Makefile (gcc, no GPU needed)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return os.path.join(_HERE, "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        src = os.path.join(_HERE, "mwu_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(path)
        vp, i64, i32, d = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.oracle_mwu.argtypes = [i32, vp, vp, vp, i64, i64, vp, i64, i32, i32, i32, i32, i32, i32,
                                 i32, i32, vp, vp, ctypes.c_char_p, i32]
        L.oracle_mwu.restype = i32
        L.oracle_mwu_stats.argtypes = [i32, vp, vp, vp, i64, i64, vp, i64, i32, vp, vp, vp, vp]
        L.oracle_mwu_stats.restype = i32
        L.oracle_group_mean.argtypes = [i32, vp, vp, vp, i64, i64, vp, i64, i32, i32, i32, vp]
        L.oracle_group_mean.restype = i32
        L.oracle_p_asymptotic.argtypes = [d, d, d, d, d, i32]
        L.oracle_p_asymptotic.restype = d
        L.oracle_p_exact_reference.argtypes = [d, i64, i64]
        L.oracle_p_exact_reference.restype = d
        L.oracle_p_asymptotic_fast_array.argtypes = [vp, vp, vp, vp, d, i32, i64, vp]
        L.oracle_p_asymptotic_fast_array.restype = None
        L.oracle_max_threads.argtypes = []
        L.oracle_max_threads.restype = i32
        _LIB = L
    return _LIB


def _prep(data, indices, indptr, group_id):
    data = np.ascontiguousarray(data)
    if data.dtype not in DTYPE_CODES:
        raise RuntimeError("Unsupported dtype for data")
    indices = np.ascontiguousarray(indices, dtype=np.int64)
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    group_id = np.ascontiguousarray(group_id, dtype=np.int32)
    return data, indices, indptr, group_id


def mannwhitneyu(data, indices, indptr, group_id, n_targets, ref_sorted=False, tar_sorted=False,
                 tie_correction=True, use_continuity=False, zero_handling=0, alternative=2,
                 method=2, threads=-1):
    data, indices, indptr, group_id = _prep(data, indices, indptr, group_id)
    R, C = group_id.size, indptr.size - 1
    n = C * max(int(n_targets), 0)
    U1 = np.zeros(max(n, 1), np.float64)
    P = np.ones(max(n, 1), np.float64)
    err = ctypes.create_string_buffer(256)
    st = lib().oracle_mwu(DTYPE_CODES[data.dtype], data.ctypes.data, indices.ctypes.data,
                          indptr.ctypes.data, R, C, group_id.ctypes.data, int(n_targets),
                          int(ref_sorted), int(tar_sorted), int(tie_correction), int(use_continuity),
                          int(zero_handling), int(alternative), int(method), int(threads),
                          U1.ctypes.data, P.ctypes.data, err, 256)
    if st != 0:
        raise RuntimeError(err.value.decode())
    return U1[:n], P[:n]


def p_asymptotic_fast(U1, n1, n2, tie_sum, cc, alternative):
    """The reference's fast_norm p-values (scalar form) from per-test statistics."""
    arrs = [np.ascontiguousarray(np.asarray(a, dtype=np.float64)).reshape(-1) for a in (U1, n1, n2, tie_sum)]
    out = np.empty_like(arrs[0])
    lib().oracle_p_asymptotic_fast_array(*[a.ctypes.data for a in arrs], ctypes.c_double(cc),
                                         int(alternative), arrs[0].size, out.ctypes.data)
    return out


def mwu_stats(data, indices, indptr, group_id, n_targets, zero_handling):
    """(U1, n1, n2, tie_sum) gene-major, tie_sum before the tie_correction mask."""
    data, indices, indptr, group_id = _prep(data, indices, indptr, group_id)
    R, C = group_id.size, indptr.size - 1
    n = max(C * int(n_targets), 1)
    out = [np.zeros(n, np.float64) for _ in range(4)]
    lib().oracle_mwu_stats(DTYPE_CODES[data.dtype], data.ctypes.data, indices.ctypes.data,
                           indptr.ctypes.data, R, C, group_id.ctypes.data, int(n_targets),
                           int(zero_handling), *[o.ctypes.data for o in out])
    return tuple(o[:C * int(n_targets)] for o in out)


def group_mean(data, indices, indptr, group_id, n_groups, include_zeros=True, threads=-1,
               use_kahan=False):
    data, indices, indptr, group_id = _prep(data, indices, indptr, group_id)
    R, C = group_id.size, indptr.size - 1
    out = np.zeros(max(C * int(n_groups), 1), np.float64)
    lib().oracle_group_mean(DTYPE_CODES[data.dtype], data.ctypes.data, indices.ctypes.data,
                            indptr.ctypes.data, R, C, group_id.ctypes.data, int(n_groups),
                            int(include_zeros), int(use_kahan), int(threads), out.ctypes.data)
    return out[:C * int(n_groups)]


def p_asymptotic(U1, n1, n2, tie_sum, cc, alternative):
    return lib().oracle_p_asymptotic(float(U1), float(n1), float(n2), float(tie_sum), float(cc),
                                     int(alternative))


def p_exact_reference(U, n1, n2):
    return lib().oracle_p_exact_reference(float(U), int(n1), int(n2))


def max_threads() -> int:
    return int(lib().oracle_max_threads())
