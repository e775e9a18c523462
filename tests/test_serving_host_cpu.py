"""Host side of the serving harness on the CPU: the query generator and the Poisson driver.

random_query draws the serving workload's groupings (reference of 1k-50k cells, 1-200
targets of 20-5,000 cells, log-uniform, cells without replacement). Every query it returns
must be answerable: each group keeps at least 2 cells, groups do not overlap, and the
cells fit the matrix, also when the draw has to shrink to fit a small matrix. poisson_run is
driven here with a stand-in server (no GPU): it must submit every planned query once, count
the tests of each, and report the percentiles of the latencies the queries report.
"""
import numpy as np
import pytest

from hpdex_gb300.serving import poisson_run, random_query


@pytest.mark.parametrize("n_rows", [1_000_000, 200_000, 50_000, 5_000, 600, 402])
def test_random_query_groups_are_valid(n_rows):
    for seed in range(60):
        rng = np.random.default_rng(seed)
        gid, T = random_query(rng, n_rows)
        assert gid.dtype == np.int32 and gid.size == n_rows
        assert 1 <= T <= 200
        assert gid.min() >= -1 and gid.max() <= T
        counts = np.bincount(gid[gid >= 0], minlength=T + 1)
        assert counts.size == T + 1
        assert counts.min() >= 2, (seed, T, counts.min())
        assert counts[0] <= 50_000 and counts[1:].max() <= 5_000


def test_random_query_unshrunk_sizes_follow_the_ranges():
    """On a matrix large enough for every draw, the sizes are the drawn ones."""
    for seed in range(40):
        gid, T = random_query(np.random.default_rng(seed), 1_000_000)
        counts = np.bincount(gid[gid >= 0], minlength=T + 1)
        assert 1_000 <= counts[0] <= 50_000
        assert counts[1:].min() >= 20 and counts[1:].max() <= 5_000


def test_random_query_rejects_a_matrix_too_small_for_its_groups():
    rng = np.random.default_rng(0)
    with pytest.raises(ValueError):
        random_query(rng, 3, targets_range=(5, 5))


class _Mat:
    def __init__(self, n_cols):
        self.n_cols = n_cols


class _Query:
    def __init__(self, latency):
        self.latency_ms = None
        self._lat = latency

    def result(self):
        self.latency_ms = self._lat
        return None, None


class _StandInServer:
    """Duck-types the part of Server that poisson_run uses."""

    def __init__(self, n_cols):
        self._mats = [_Mat(c) for c in n_cols]
        self.submitted = []
        self._rng = np.random.default_rng(7)

    def submit(self, mid, gid, T, **options):
        self.submitted.append((mid, int(T), int((gid >= 0).sum()), options))
        return _Query(float(self._rng.uniform(1.0, 50.0)))

    def stats(self):
        return {"completed": len(self.submitted), "batches": 1, "busy_ms": 0.0}


def test_poisson_run_submits_every_query_and_reports_percentiles():
    srv = _StandInServer([30, 70])
    rows = {0: 60_000, 1: 80_000}
    out = poisson_run(srv, [0, 1], rows, rate_qps=1e6, n_queries=40, seed=3)
    assert len(srv.submitted) == 40
    assert out["queries"] == 40 and out["completed"] == 40
    assert out["tests"] == sum(T * srv._mats[mid].n_cols for mid, T, _, _ in srv.submitted)
    lat = np.random.default_rng(7).uniform(1.0, 50.0, size=40)
    assert out["p50_ms"] == pytest.approx(np.percentile(lat, 50))
    assert out["p99_ms"] == pytest.approx(np.percentile(lat, 99))
    assert out["mean_ms"] == pytest.approx(lat.mean())
    assert all(o == dict(zero_handling="min", use_continuity=True, tie_correction=True)
               for _, _, _, o in srv.submitted)
    # the same seed plans the same queries
    srv2 = _StandInServer([30, 70])
    poisson_run(srv2, [0, 1], rows, rate_qps=1e6, n_queries=40, seed=3)
    assert [s[:3] for s in srv2.submitted] == [s[:3] for s in srv.submitted]
