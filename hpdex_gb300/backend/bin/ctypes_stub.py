"""The smallest binding a maintainer of the reference would add to run its Python layer on
this library: ctypes over the C ABI (include/hpdex_gb300.h), no pybind11.

`kernel.mannwhitneyu` of the reference (src/cpp/module.cpp:196-228) becomes `mannwhitneyu`
below, with the same arguments and errors; results are (n_targets, n_genes) arrays. The full
shim, `hpdex_gb300/backend/bin/kernel.py`, is this core plus `group_mean`, int32 row ids passed
through and page-locked result buffers.
"""
import ctypes

import numpy as np


class Opt(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("ref_sorted", "tar_sorted", "tie_correction",
                "use_continuity", "fast_norm", "zero_handling", "alternative", "method",
                "exact_variant")]


DTYPE = {np.dtype(t): i for i, t in enumerate(("int8", "uint8", "int16", "uint16", "int32",
         "uint32", "int64", "uint64", "float32", "float64"))}   # HPDEX_INT8 .. HPDEX_FLOAT64


def bind(path="libhpdex_gb300.so"):
    """Loads the library and returns (lib, mannwhitneyu)."""
    lib = ctypes.CDLL(path)
    P, I64, I32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
    lib.hpdex_mannwhitneyu.argtypes = [I32, P, P, P, I64, I64, I64, P, I64, ctypes.POINTER(Opt),
                                       I32, P, P]   # without argtypes ctypes would pass C ints
    lib.hpdex_mannwhitneyu.restype = ctypes.c_int
    lib.hpdex_last_error.restype = ctypes.c_char_p

    def mannwhitneyu(data, indices, indptr, group_id, n_targets, ref_sorted=False,
                     tar_sorted=False, tie_correction=True, use_continuity=False, fast_norm=True,
                     zero_handling=0, alternative=2, method=2, threads=-1, layout="csc",
                     show_progress=False):
        if np.dtype(data.dtype) not in DTYPE:
            raise RuntimeError("Unsupported dtype for data")
        data = np.ascontiguousarray(data)
        indices = np.ascontiguousarray(indices, dtype=np.int64)
        indptr = np.ascontiguousarray(indptr, dtype=np.int64)
        group_id = np.ascontiguousarray(group_id, dtype=np.int32)
        o = Opt(int(ref_sorted), int(tar_sorted), int(tie_correction), int(use_continuity),
                int(fast_norm), zero_handling, alternative, method, 0)
        C = len(indptr) - 1
        U1 = np.empty((n_targets, C))
        P_ = np.empty((n_targets, C))
        st = lib.hpdex_mannwhitneyu(DTYPE[data.dtype], data.ctypes.data, indices.ctypes.data,
                                    indptr.ctypes.data, len(group_id), C, data.size,
                                    group_id.ctypes.data, n_targets, ctypes.byref(o), threads,
                                    U1.ctypes.data, P_.ctypes.data)
        if st:
            raise RuntimeError(lib.hpdex_last_error().decode())
        return U1, P_

    return lib, mannwhitneyu
