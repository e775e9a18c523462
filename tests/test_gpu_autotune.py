"""GPU: the plan's layout tuner times every candidate rank-kernel layout (run counters in shared
or global memory, bucket table of 2^13 or 2^12 entries), keeps the fastest and leaves the
results unchanged, bit for bit."""
import numpy as np
import pytest

from test_gpu_large_columns import COLUMNS, _workload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_targets", [12, 1200])
def test_autotune_keeps_the_fastest_layout_and_the_results(n_targets):
    from hpdex_gb300.resident import BATCHED, ResidentMatrix
    rng = np.random.default_rng(23)
    sizes = list(rng.integers(20, 90, size=n_targets)) if n_targets > 12 else \
        [500, 800, 1200, 2000, 3000, 4500, 6000, 700, 650, 5200, 900, 3300]
    w = _workload(7, 120_000, COLUMNS, 20_000, sizes)
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    try:
        plan = M.plan(w.group_id, w.n_targets, zero_handling="min", use_continuity=True)
        plan.run(BATCHED)
        U1a, Pa = plan.download()
        tuned = plan.autotune(reps=2)
        assert tuned["run_counters"] in ("shared", "global") and tuned["bucket_bits"] in (12, 13)
        ms = tuned["ms"]
        assert len(ms) == 4 and all(t > 0.0 for t in ms.values())
        assert ms[f"{tuned['run_counters']}/2^{tuned['bucket_bits']}"] == min(ms.values())
        plan.run(BATCHED)  # the kept layout
        U1b, Pb = plan.download()
        np.testing.assert_array_equal(U1b, U1a)
        np.testing.assert_array_equal(Pb, Pa)
        plan.close()
    finally:
        M.close()


def test_autotune_reports_the_plans_error():
    """A plan whose runs fail (a reference of 3 cells under zero_handling=none: most genes store
    fewer than 2 of them) makes the tuner raise the run's error, as a run would."""
    from hpdex_gb300.resident import BATCHED, ResidentMatrix
    from hpdex_gb300 import synthetic
    w = synthetic.umi_counts(seed=42, n_rows=8_000, n_cols=50, n_targets=5)
    gid = np.full(w.n_rows, -1, np.int32)
    gid[:3] = 0
    gid[3:6] = 1
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    try:
        plan = M.plan(gid, 1, zero_handling="none")
        with pytest.raises(RuntimeError) as e_run:
            plan.run(BATCHED)
        with pytest.raises(RuntimeError) as e_tune:
            plan.autotune(reps=1)
        assert str(e_tune.value) == str(e_run.value)
        assert "Sample too small" in str(e_tune.value)
        plan.close()
    finally:
        M.close()
