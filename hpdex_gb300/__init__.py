"""hpdex_gb300 -- GB300 (sm_103a) Mann-Whitney U differential-expression backend.

Drop-in for AI4Cell/hpdex's MWU path: `backend.mannwhitneyu`, `backend.group_mean`,
`backend.bin.kernel` and `parallel_differential_expression` keep the reference's
signatures; the compute runs in hand-written CUDA through the C ABI of
libhpdex_gb300.so (include/hpdex_gb300.h). There is no CPU fallback.
"""
from .backend import group_mean, mannwhitneyu  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # the DE driver and the resident API load lazily (pandas only for the AnnData front-end)
    if name in ("parallel_differential_expression", "differential_expression", "pde"):
        from . import de
        return de.parallel_differential_expression if name in ("parallel_differential_expression", "pde") else de.differential_expression
    if name in ("ResidentMatrix", "Plan"):
        from . import resident
        return getattr(resident, name)
    if name == "release_cached_memory":
        from ._lib import release_cached_memory
        return release_cached_memory
    raise AttributeError(name)


__all__ = ["mannwhitneyu", "group_mean", "parallel_differential_expression",
           "differential_expression", "ResidentMatrix", "Plan", "release_cached_memory"]
