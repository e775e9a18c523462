"""Python wrappers with the reference's signatures (AI4Cell/hpdex
src/hpdex/backend/mannwhitneyu_.py:28-127): scipy CSR/CSC in, string options mapped to the
binding's integers, indptr cast to int64 (indices to int64 unless they are int32) and group_id
to int32."""
from __future__ import annotations

from typing import Literal

import numpy as np
import scipy.sparse

from .bin import kernel

__all__ = ["mannwhitneyu", "group_mean"]

_zero_handling_map = {"none": 0, "min": 1, "max": 2, "mix": 3}
_alternative_map = {"less": 0, "greater": 1, "two-sided": 2}
_method_map = {"exact": 1, "asymptotic": 2}


def _sparse_parts(sparse_matrix, group_id):
    if not isinstance(sparse_matrix, (scipy.sparse.csr_matrix, scipy.sparse.csc_matrix)):
        raise ValueError("sparse_matrix must be CSR or CSC")
    if isinstance(sparse_matrix, scipy.sparse.csc_matrix):
        R = sparse_matrix.shape[0]
    else:
        R = sparse_matrix.shape[1]
    if group_id.ndim != 1 or len(group_id) != R:
        raise ValueError(f"group_id must be 1D with length {R} (rows of CSC / cols of CSR)")
    group_id = group_id.astype(np.int32, copy=False)
    data = sparse_matrix.data
    # int32 row ids stay int32: the binding takes them as they are (the reference casts to
    # int64 here; the results are the same)
    indices = sparse_matrix.indices
    if indices.dtype != np.int32:
        indices = indices.astype(np.int64, copy=False)
    indptr = sparse_matrix.indptr.astype(np.int64, copy=False)
    layout = "csc" if isinstance(sparse_matrix, scipy.sparse.csc_matrix) else "csr"
    return data, indices, indptr, group_id, layout


def mannwhitneyu(
    sparse_matrix,
    group_id: np.ndarray,
    n_targets: int,
    ref_sorted: bool = False,
    tar_sorted: bool = False,
    tie_correction: bool = True,
    use_continuity: bool = False,
    fast_norm: bool = False,
    zero_handling: Literal["none", "min", "max", "mix"] = "mix",
    alternative: Literal["less", "greater", "two-sided"] = "two-sided",
    method: Literal["exact", "asymptotic"] = "asymptotic",
    threads: int = -1,
    show_progress: bool = False,
    exact_variant: Literal["reference", "mwu_null"] = "reference",
) -> tuple[np.ndarray, np.ndarray]:
    """Mann-Whitney U test on a sparse CSR/CSC matrix (multi-group).

    Returns (U1, P), float64 arrays of shape (n_targets, n_genes). `exact_variant`
    (method="exact" only) chooses between the reference's exact p-values ("reference")
    and the true MWU null distribution ("mwu_null")."""
    data, indices, indptr, group_id, layout = _sparse_parts(sparse_matrix, group_id)
    return kernel.mannwhitneyu(
        data=data, indices=indices, indptr=indptr, group_id=group_id, n_targets=n_targets,
        ref_sorted=ref_sorted, tar_sorted=tar_sorted, tie_correction=tie_correction,
        use_continuity=use_continuity, fast_norm=fast_norm,
        zero_handling=_zero_handling_map[zero_handling],
        alternative=_alternative_map[alternative], method=_method_map[method],
        threads=threads, layout=layout, show_progress=show_progress,
        exact_variant={"reference": 0, "mwu_null": 1}[exact_variant])


def group_mean(
    sparse_matrix,
    group_id: np.ndarray,
    n_groups: int,
    include_zeros: bool = True,
    use_kahan: bool = False,
    threads: int = -1,
) -> np.ndarray:
    """Group-wise mean for each feature, flat [gene * n_groups + g]."""
    data, indices, indptr, group_id, layout = _sparse_parts(sparse_matrix, group_id)
    return kernel.group_mean(data=data, indices=indices, indptr=indptr, group_id=group_id,
                             n_groups=n_groups, include_zeros=include_zeros, threads=threads,
                             use_kahan=use_kahan, layout=layout)
