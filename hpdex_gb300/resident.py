"""HBM-resident matrices and plans: the reference call split into upload, run, download.

    M = ResidentMatrix(data, indices, indptr, n_rows)      # CSC, stays on the GPU
    plan = M.plan(group_id, n_targets, zero_handling="min", use_continuity=True)
    plan.run()                    # batched form: persistent kernel + work queue, CUDA graph
    U1, P = plan.download()       # (n_targets, n_genes) float64
The same plan can run again (graph replay) or in the plain form (one launch per gene).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_ZH = {"none": 0, "min": 1, "max": 2, "mix": 3}
_ALT = {"less": 0, "greater": 1, "two-sided": 2}
_METHOD = {"exact": 1, "asymptotic": 2}

BATCHED, PLAIN = 0, 1


def make_options(tie_correction=True, use_continuity=False, zero_handling="mix",
                 alternative="two-sided", method="asymptotic", exact_variant="reference",
                 fast_norm=False):
    o = _lib.MwuOptions()
    o.fast_norm = int(bool(fast_norm))
    o.tie_correction = int(bool(tie_correction))
    o.use_continuity = int(bool(use_continuity))
    o.zero_handling = _ZH[zero_handling] if isinstance(zero_handling, str) else int(zero_handling)
    o.alternative = _ALT[alternative] if isinstance(alternative, str) else int(alternative)
    o.method = _METHOD[method] if isinstance(method, str) else int(method)
    o.exact_variant = {"reference": 0, "mwu_null": 1}.get(exact_variant, exact_variant)
    return o


class ResidentMatrix:
    def __init__(self, data, indices, indptr, n_rows):
        data = np.ascontiguousarray(data)
        if data.dtype.name not in _lib.DTYPE_CODES:
            raise RuntimeError("Unsupported dtype for data")
        indices = np.asarray(indices)
        idx32 = indices.dtype == np.int32  # int32 row ids are uploaded as they are
        indices = np.ascontiguousarray(indices, dtype=np.int32 if idx32 else np.int64)
        indptr = np.ascontiguousarray(indptr, dtype=np.int64)
        self.n_rows = int(n_rows)
        self.n_cols = indptr.size - 1
        self.nnz = data.size
        self.dtype = data.dtype
        h = ctypes.c_void_p()
        create = _lib.lib().hpdex_matrix_create_idx32 if idx32 else _lib.lib().hpdex_matrix_create
        _lib.check(create(_lib.DTYPE_CODES[data.dtype.name], data.ctypes.data, indices.ctypes.data,
                          indptr.ctypes.data, self.n_rows, self.n_cols, self.nnz, ctypes.byref(h)))
        self._h = h

    @classmethod
    def from_scipy(cls, X):
        """A cells x genes scipy matrix: CSC as is, CSR transposed on the device."""
        import scipy.sparse as sp
        if isinstance(X, sp.csr_matrix):
            return cls.from_csr(X.data, X.indices, X.indptr, X.shape[0], X.shape[1])
        X = X if isinstance(X, sp.csc_matrix) else sp.csc_matrix(X)
        return cls(X.data, X.indices, X.indptr, X.shape[0])

    @classmethod
    def from_csr(cls, data, indices, indptr, n_rows, n_cols):
        """A cells x genes CSR (AnnData's native layout), transposed to CSC on the device."""
        self = cls.__new__(cls)
        data = np.ascontiguousarray(data)
        if data.dtype.name not in _lib.DTYPE_CODES:
            raise RuntimeError("Unsupported dtype for data")
        indices = np.asarray(indices)
        idx32 = indices.dtype == np.int32  # int32 gene ids are uploaded as they are
        indices = np.ascontiguousarray(indices, dtype=np.int32 if idx32 else np.int64)
        indptr = np.ascontiguousarray(indptr, dtype=np.int64)
        self.n_rows, self.n_cols, self.dtype = int(n_rows), int(n_cols), data.dtype
        if indptr.size != self.n_rows + 1:
            raise ValueError("indptr must hold n_rows + 1 entries")
        h = ctypes.c_void_p()
        create = (_lib.lib().hpdex_matrix_create_csr_idx32 if idx32
                  else _lib.lib().hpdex_matrix_create_csr)
        _lib.check(create(_lib.DTYPE_CODES[data.dtype.name], data.ctypes.data, indices.ctypes.data,
                          indptr.ctypes.data, self.n_rows, self.n_cols, data.size, ctypes.byref(h)))
        self._h = h
        self.nnz = self._info()[2]
        return self

    @classmethod
    def from_device(cls, data_ptr: int, rows_ptr: int, indptr, n_rows: int, dtype):
        """A matrix whose values (`dtype`) and int32 row ids are already in device memory at
        data_ptr / rows_ptr (copied into the library's buffers); indptr is a host array."""
        self = cls.__new__(cls)
        dtype = np.dtype(dtype)
        if dtype.name not in _lib.DTYPE_CODES:
            raise RuntimeError("Unsupported dtype for data")
        indptr = np.ascontiguousarray(indptr, dtype=np.int64)
        self.n_rows, self.n_cols, self.dtype = int(n_rows), indptr.size - 1, dtype
        self.nnz = int(indptr[-1])
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().hpdex_matrix_create_device(_lib.DTYPE_CODES[dtype.name], int(data_ptr),
                                                         int(rows_ptr), indptr.ctypes.data,
                                                         self.n_rows, self.n_cols, self.nnz,
                                                         ctypes.byref(h)))
        self._h = h
        return self

    def _info(self):
        v = [ctypes.c_int64() for _ in range(4)]
        _lib.check(_lib.lib().hpdex_matrix_info(self._h, *[ctypes.byref(x) for x in v]))
        return [x.value for x in v]

    def group_mean(self, group_id, n_groups, include_zeros=True):
        """Per (gene, group) means, flat [gene * n_groups + g] (the reference's layout)."""
        gid = np.ascontiguousarray(np.asarray(group_id), dtype=np.int32)
        if gid.size != self.n_rows:
            raise ValueError(f"group_id has {gid.size} entries, the matrix {self.n_rows} rows")
        out = np.zeros(max(self.n_cols, 0) * max(int(n_groups), 0), np.float64)
        _lib.check(_lib.lib().hpdex_matrix_group_mean(self._h, gid.ctypes.data, int(n_groups),
                                                      int(bool(include_zeros)), out.ctypes.data))
        return out

    def device_bytes(self) -> int:
        v = [ctypes.c_int64() for _ in range(4)]
        _lib.check(_lib.lib().hpdex_matrix_info(self._h, *[ctypes.byref(x) for x in v]))
        return v[3].value

    def plan(self, group_id, n_targets, **options) -> "Plan":
        return Plan(self, group_id, n_targets, make_options(**options))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.lib().hpdex_matrix_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    def __init__(self, matrix: ResidentMatrix, group_id, n_targets, options):
        self.matrix = matrix
        gid = np.ascontiguousarray(group_id, dtype=np.int32)
        if gid.size != matrix.n_rows:
            raise ValueError(f"group_id must have length {matrix.n_rows}")
        self.n_targets = int(n_targets)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().hpdex_plan_create(matrix._h, gid.ctypes.data, self.n_targets,
                                                ctypes.byref(options), ctypes.byref(h)))
        self._h = h

    def run(self, mode: int = BATCHED) -> None:
        _lib.check(_lib.lib().hpdex_plan_run(self._h, int(mode)))

    def set_fused_pvalues(self, on: bool) -> None:
        """Asymptotic p-values inside the rank kernel (default) or in a separate kernel."""
        _lib.check(_lib.lib().hpdex_plan_set_fused_pvalues(self._h, int(bool(on))))

    def set_bucket_bits(self, bits: int) -> None:
        """Diagnostic: the rank kernel's bucket table of 2**bits entries (9..13); the results do
        not change."""
        _lib.check(_lib.lib().hpdex_plan_set_bucket_bits(self._h, int(bits)))

    def set_histogram(self, on: bool) -> None:
        """Per-gene histogram path for small-integer values (default) or the bucket path for
        every gene; the results are the same."""
        _lib.check(_lib.lib().hpdex_plan_set_histogram(self._h, int(bool(on))))

    def set_run_counters(self, mode: int) -> None:
        """Diagnostic: the rank kernel's per-warp run counters in shared memory (1), in global
        memory (0, rounds by warp match) or placed automatically (-1, the default: shared up to
        1,024 groups); results do not change."""
        _lib.check(_lib.lib().hpdex_plan_set_run_counters(self._h, int(mode)))

    def autotune(self, reps: int = 3) -> dict:
        """Times the plan under each candidate rank-kernel layout (run counters in shared or
        global memory, bucket table of 2^13 or 2^12 entries) and keeps the fastest; results do
        not change. Returns the choice and the mean time of every candidate."""
        mode, bits = ctypes.c_int32(), ctypes.c_int32()
        ms = (ctypes.c_float * 4)()
        _lib.check(_lib.lib().hpdex_plan_autotune(self._h, int(reps), ctypes.byref(mode),
                                                  ctypes.byref(bits), ms))
        names = [("shared", 13), ("shared", 12), ("global", 13), ("global", 12)]
        return {"run_counters": "shared" if mode.value == 1 else "global",
                "bucket_bits": bits.value,
                "ms": {f"{c}/2^{b}": round(float(t), 4) for (c, b), t in zip(names, ms)}}

    def set_drain_wait(self, on: bool) -> None:
        """Diagnostic: on makes a warp of the rank kernel wait a bounded number of polls for a
        large bucket another warp is still listing (off, the default, leaves it to the pass after
        the block barrier); results do not change."""
        _lib.check(_lib.lib().hpdex_plan_set_drain_wait(self._h, int(bool(on))))

    def download(self):
        C = self.matrix.n_cols
        U1 = np.empty((self.n_targets, C), np.float64)
        P = np.empty((self.n_targets, C), np.float64)
        _lib.check(_lib.lib().hpdex_plan_download(self._h, U1.ctypes.data, P.ctypes.data))
        return U1, P

    def timings(self):
        """(total_ms, rank_ms, pvalue_ms), kernel launches of the last run."""
        ms = (ctypes.c_float * 3)()
        n = ctypes.c_int32()
        _lib.check(_lib.lib().hpdex_plan_timings(self._h, ms, ctypes.byref(n)))
        return (ms[0], ms[1], ms[2]), n.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.lib().hpdex_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
