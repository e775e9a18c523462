"""GPU: the deep tail of the p-values and the ranking of P and FDR.

The strongly shifted workload (hpdex_gb300.synthetic.extreme_shift: 20,000 reference cells
against targets of 3,000 / 1,000 / 3,000 cells, |z| up to ~90) drives p-values through the
subnormal range, where the reference still reports nonzero values (glibc's erfc) down to
4.9e-324. Against the reference's stored outputs (tests/golden/extreme_shift_outputs.npz):
- U1 bit-exact;
- P: zero exactly where the reference's is zero, else within 1e-12 relative with no absolute
  floor (below 4.9e-312 that is equality on the subnormal grid);
- the ranking: the stable argsort of the device's P equals that of the reference's P, and the
  BH FDR of the device (hpdex_bh_fdr on its own P) ranks the tests as scipy's BH of the
  reference's P does.
The device's erfc is also compared directly with the host C library's erfc (the function the
reference calls) on the tail [26.5, 27.3] and beyond.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_deep_tail_cpu import libm_erfc, workload_digest

pytestmark = pytest.mark.gpu

ALT = {0: "less", 1: "greater", 2: "two-sided"}


@pytest.fixture(scope="module")
def extreme():
    from hpdex_gb300 import synthetic
    w = synthetic.extreme_shift()
    z = np.load(os.path.join(GOLDEN, "extreme_shift_outputs.npz"))
    assert str(z["digest"]) == workload_digest(w), "extreme_shift() no longer reproduces its inputs"
    return w, z


def reference_tm(z, key, w):
    """Reference output (gene-major, flat) as (n_targets, n_genes)."""
    return z[key].reshape(w.n_cols, w.n_targets).T


def assert_tail_close(P, Pref):
    zero = Pref == 0.0
    assert np.array_equal(P[zero], Pref[zero]), "p-values nonzero where the reference's are 0"
    nz = ~zero
    rel = np.abs(P[nz] - Pref[nz]) / Pref[nz]
    assert rel.max() <= 1e-12, f"max rel err {rel.max():.3e} at reference p {Pref[nz][np.argmax(rel)]:.3e}"


def test_device_erfc_equals_c_library_in_the_tail():
    from hpdex_gb300 import _lib
    erfc = libm_erfc()
    rng = np.random.default_rng(4)
    x = np.concatenate([rng.uniform(26.5, 27.3, 200_000), np.linspace(26.0, 28.0, 20_001),
                        -rng.uniform(26.5, 27.3, 1000), [np.inf, -np.inf]])
    out = np.empty_like(x)
    _lib.check(_lib.lib().hpdex_selftest_erfc_values(x.ctypes.data, x.size, out.ctypes.data))
    ref = np.array([erfc(float(v)) for v in x])
    assert np.array_equal(out == 0.0, ref == 0.0)
    nz = ref != 0.0
    err = np.abs(out[nz] - ref[nz])
    assert np.all(err <= np.maximum(1e-12 * ref[nz], 5e-324)), err.max()
    deep = nz & (ref < 1e-311)
    assert deep.sum() > 100_000
    # equal on the coarse part of the grid, but for rare one-step flips of exp(a)'s rounding
    assert (out[deep] != ref[deep]).sum() <= deep.sum() // 10_000


@pytest.mark.parametrize("alt", [0, 1, 2])
def test_one_shot_deep_tail_matches_reference(extreme, alt):
    from hpdex_gb300.backend.bin import kernel
    w, z = extreme
    U1, P = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                                tie_correction=True, use_continuity=True, zero_handling=1,
                                alternative=alt, fast_norm=False)
    np.testing.assert_array_equal(U1, reference_tm(z, f"U1_alt{alt}", w))
    assert_tail_close(P, reference_tm(z, f"P_alt{alt}", w))


@pytest.mark.parametrize("fused", [True, False])
def test_resident_deep_tail_matches_reference(extreme, fused):
    from hpdex_gb300.resident import BATCHED, ResidentMatrix
    w, z = extreme
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    try:
        plan = M.plan(w.group_id, w.n_targets, zero_handling="min", alternative="two-sided",
                      use_continuity=True, tie_correction=True)
        plan.set_fused_pvalues(fused)
        plan.run(BATCHED)
        U1, P = plan.download()
        plan.close()
    finally:
        M.close()
    np.testing.assert_array_equal(U1, reference_tm(z, "U1_alt2", w))
    assert_tail_close(P, reference_tm(z, "P_alt2", w))


def test_ranking_of_p_and_fdr_equals_reference(extreme):
    from scipy.stats import false_discovery_control
    from hpdex_gb300._lib import bh_fdr
    from hpdex_gb300.backend.bin import kernel
    w, z = extreme
    _, P = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, w.n_targets,
                               tie_correction=True, use_continuity=True, zero_handling=1,
                               alternative=2, fast_norm=False)
    Pref = np.ascontiguousarray(reference_tm(z, "P_alt2", w))
    p, pr = P.reshape(-1), Pref.reshape(-1)
    np.testing.assert_array_equal(np.argsort(p, kind="stable"), np.argsort(pr, kind="stable"))
    fdr, fdr_ref = bh_fdr(p), false_discovery_control(pr, method="bh")
    np.testing.assert_array_equal(np.argsort(fdr, kind="stable"), np.argsort(fdr_ref, kind="stable"))
