"""Differential expression driver with the reference's output schema (AI4Cell/hpdex
src/hpdex/de.py:35-198).

`parallel_differential_expression(adata, ...)` keeps the reference signature and returns a
pandas DataFrame with columns target, feature, p_value, u_statistic, fold_change,
log2_fold_change, fdr. pandas/anndata are imported lazily; `differential_expression`
does the same work on plain arrays (a CSC/CSR/dense matrix and one label per cell) and
returns the seven columns as a dict of numpy arrays.

One deliberate difference: the reference pairs p_value/u_statistic with (target, feature)
labels in target-major order while its kernel writes them gene-major (de.py:159-170 vs
mannwhitneyu.cpp:959), which mislabels rows when there is more than one target. The GPU
kernel returns (n_targets, n_genes), so the flattened order matches the labels.
"""
from __future__ import annotations

import logging

import numpy as np


logger = logging.getLogger(__name__)

supported_metrics = ["wilcoxon"]
COLUMNS = ["target", "feature", "p_value", "u_statistic", "fold_change", "log2_fold_change", "fdr"]


def _bh(P: np.ndarray) -> np.ndarray:
    """BH FDR on the device: scipy.stats.false_discovery_control(P, method="bh"), as the
    reference driver calls it (de.py:174-184), with its NaN fallback on failure."""
    from ._lib import bh_fdr
    try:
        return bh_fdr(P)
    except Exception:
        logger.warning("FDR correction failed, falling back to NaN")
        return np.full_like(P, np.nan)


def _select_groups(labels, reference, groups, min_samples):
    uniq = list(dict.fromkeys(labels.tolist()))  # order of first appearance (pandas unique)
    if groups is None:
        groups = [g for g in uniq if g != reference]
    else:
        groups = [g for g in groups if g in uniq and g != reference]
    if reference not in uniq:
        raise ValueError(f"Reference `{reference}` not found")
    if not groups:
        raise ValueError("No valid target groups found")
    valid = []
    for g in groups:
        count = int(np.sum(labels == g))
        if count >= min_samples:
            valid.append(g)
        else:
            logger.warning(f"Group `{g}` has only {count} samples, skipping")
    return valid


def differential_expression(X, labels, reference, features=None, groups=None,
                            metric="wilcoxon", tie_correction=True, use_continuity=True,
                            min_samples=2, threads=-1, clip_value=20.0, show_progress=False):
    """Array-level DE: X is cells x genes (CSC, CSR or dense), labels one per cell."""
    if metric not in supported_metrics:
        raise ValueError(f"Unsupported metric: {metric}; supported: {supported_metrics}")
    labels = np.asarray(labels, dtype=object)
    groups = _select_groups(labels, reference, groups, min_samples)
    n_genes = X.shape[1]
    features = np.asarray(features if features is not None else np.arange(n_genes), dtype=object)
    if not groups:
        return {c: np.zeros(0, dtype=object if c in ("target", "feature") else np.float64)
                for c in COLUMNS}
    group_map = {reference: 0}
    for i, g in enumerate(groups):
        group_map[g] = i + 1
    group_id = np.full(labels.size, -1, dtype=np.int32)
    for g, idx in group_map.items():
        group_id[labels == g] = idx
    n_targets = len(groups)

    # one upload serves the means and the tests: CSC as is, a cells x genes CSR transposed on
    # the device (the reference converts with tocsc() on the host, de.py:106-107)
    from ._lib import fold_change
    from .resident import ResidentMatrix
    M = ResidentMatrix.from_scipy(X)
    # fold change and log2 fold change on the device from the group means (de.py:138-142)
    means = M.group_mean(group_id, n_targets + 1, include_zeros=True)
    fold, log2fold = fold_change(means, n_genes, n_targets + 1, clip_value)

    plan = M.plan(group_id, n_targets, use_continuity=use_continuity,
                  tie_correction=tie_correction, zero_handling="min")
    plan.run()
    U1, P = plan.download()
    U1 = np.asarray(U1).reshape(-1)
    P = np.asarray(P).reshape(-1)
    return {
        "target": np.repeat(np.asarray(groups, dtype=object), n_genes),
        "feature": np.tile(features, n_targets),
        "p_value": P,
        "u_statistic": U1,
        "fold_change": fold.reshape(-1),
        "log2_fold_change": log2fold.reshape(-1),
        "fdr": _bh(P),
    }


def parallel_differential_expression(adata, groupby_key: str, reference, groups=None,
                                     metric: str = "wilcoxon", tie_correction: bool = True,
                                     use_continuity: bool = True, min_samples: int = 2,
                                     threads: int = -1, clip_value: float = 20.0,
                                     show_progress: bool = True):
    """AnnData front-end with the reference's signature; returns a pandas DataFrame."""
    import pandas as pd  # lazy: only this front-end needs pandas

    if metric not in supported_metrics:
        raise ValueError(f"Unsupported metric: {metric}; supported: {supported_metrics}")
    if groupby_key not in adata.obs.columns:
        raise ValueError(f"Groupby key `{groupby_key}` not found in adata.obs")
    obs = adata.obs.copy()
    if reference is None:
        obs[groupby_key] = obs[groupby_key].cat.add_categories("non-targeting")
        obs[groupby_key] = obs[groupby_key].fillna("non-targeting")
        reference = "non-targeting"
    labels = np.asarray(obs[groupby_key].astype(object))
    cols = differential_expression(adata.X, labels, reference,
                                   features=np.asarray(adata.var_names, dtype=object),
                                   groups=groups, metric=metric, tie_correction=tie_correction,
                                   use_continuity=use_continuity, min_samples=min_samples,
                                   threads=threads, clip_value=clip_value,
                                   show_progress=show_progress)
    return pd.DataFrame({c: cols[c] for c in COLUMNS})
