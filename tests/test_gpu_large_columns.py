"""GPU parity on columns larger than the rank kernel's shared-memory capacity: such a column is
scattered into bucket order in global memory and ranked in slabs that a bulk copy brings into
shared memory (or, for a slab made of one oversized bucket, ranked in place). The columns mix
continuous values, heavy ties, one dominant value (a bucket above 65,535 elements), and
buckets holding many distinct keys (keys packed within a few ulps next to a far outlier)."""
from types import SimpleNamespace

import numpy as np
import pytest

from test_gpu_parity import _oracle_compare

pytestmark = pytest.mark.gpu


def _csc(columns, n_rows, rng):
    """columns: list of (density, sampler(k) -> float32 values)."""
    data, indices, indptr = [], [], [0]
    for dens, sampler in columns:
        k = int(round(dens * n_rows))
        rows = np.sort(rng.choice(n_rows, size=k, replace=False)) if k < n_rows else np.arange(n_rows)
        data.append(sampler(k).astype(np.float32))
        indices.append(rows.astype(np.int64))
        indptr.append(indptr[-1] + k)
    return np.concatenate(data), np.concatenate(indices), np.asarray(indptr, dtype=np.int64)


def _groups(rng, n_rows, ref, sizes):
    gid = np.full(n_rows, -1, dtype=np.int32)
    perm = rng.permutation(n_rows)
    gid[perm[:ref]] = 0
    o = ref
    for t, s in enumerate(sizes, start=1):
        gid[perm[o:o + s]] = t
        o += s
    return gid


def _workload(seed, n_rows, columns, ref, sizes):
    rng = np.random.default_rng(seed)
    data, indices, indptr = _csc([(d, f(rng)) for d, f in columns], n_rows, rng)
    return SimpleNamespace(data=data, indices=indices, indptr=indptr, n_rows=n_rows,
                           n_cols=indptr.size - 1, n_targets=len(sizes),
                           group_id=_groups(rng, n_rows, ref, sizes))


def _packed_ulps(rng):
    def f(k):
        base = np.float32(1.0).view(np.uint32)
        v = (base + rng.integers(0, 300, size=k).astype(np.uint32)).view(np.float32)
        v[rng.random(k) < 0.001] = 1e6  # stretches the key range: few buckets, many keys each
        return v
    return f


def _normal_with_packed(rng):
    """90% N(0,1), 10% within 300 ulps of 1.0: one bucket of ~7,500 elements and 300 keys,
    above half the shared-memory capacity, in a column that needs several slabs."""
    def f(k):
        v = rng.standard_normal(k).astype(np.float32)
        sel = rng.random(k) < 0.1
        base = np.float32(1.0).view(np.uint32)
        v[sel] = (base + rng.integers(0, 300, size=int(sel.sum())).astype(np.uint32)).view(np.float32)
        return v
    return f


COLUMNS = [
    (1.0, lambda rng: (lambda k: rng.standard_normal(k))),                      # continuous
    (0.7, lambda rng: (lambda k: rng.lognormal(0.0, 1.0, k))),                  # continuous, sparse
    (1.0, lambda rng: (lambda k: np.round(rng.standard_normal(k) * 64) / 64)),  # heavy ties
    (0.08, _packed_ulps),                                                       # impure big bucket
    (0.5, _normal_with_packed),                                                 # impure, oversized
    (0.95, lambda rng: (lambda k: np.where(rng.random(k) < 0.95, 2.0,           # dominant value
                                            rng.standard_normal(k)))),
    (1.0, lambda rng: (lambda k: np.full(k, 3.0))),                             # one value
]


@pytest.mark.parametrize("zh", ["min", "none", "mix"])
def test_large_columns_match_oracle(zh):
    sizes = [500, 800, 1200, 2000, 3000, 4500, 6000, 700, 650, 5200, 900, 3300]
    w = _workload(3, 150_000, COLUMNS, 30_000, sizes)
    assert _oracle_compare(w, zero_handling=zh) == "ok"


def test_large_columns_many_targets():
    """Small groups over a long column: most (key, group) runs hold one element."""
    rng = np.random.default_rng(9)
    sizes = list(rng.integers(20, 400, size=300))
    w = _workload(4, 120_000, COLUMNS[:5], 20_000, sizes)
    assert _oracle_compare(w, zero_handling="min") == "ok"


@pytest.mark.parametrize("fused", [True, False])
def test_drain_wait_fallback_gives_identical_results(fused):
    """Warps that resolve listed big buckets while other warps still list them either leave an
    entry not yet published to the pass after the block barrier (the default) or wait a bounded
    number of polls for it. Both must give the same doubles, in both p-value forms."""
    from hpdex_gb300.resident import BATCHED, ResidentMatrix
    sizes = [500, 800, 1200, 2000, 3000, 4500, 6000, 700, 650, 5200, 900, 3300]
    w = _workload(3, 150_000, COLUMNS, 30_000, sizes)
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    try:
        plan = M.plan(w.group_id, w.n_targets, zero_handling="min", use_continuity=True)
        plan.set_fused_pvalues(fused)
        plan.run(BATCHED)
        U1a, Pa = plan.download()
        plan.set_drain_wait(True)
        for _ in range(2):
            plan.run(BATCHED)
            U1b, Pb = plan.download()
            np.testing.assert_array_equal(U1b, U1a)
            np.testing.assert_array_equal(Pb, Pa)
        plan.close()
    finally:
        M.close()


def _signed_wide(rng):
    """Both signs over 60 decades, with subnormals, ties and values next to the signed bucket
    map's linear/log junction (signed powers of two)."""
    def f(k):
        v = rng.standard_normal(k) * 10.0 ** rng.uniform(-30, 30, k)
        v[rng.random(k) < 0.05] = 1e-42
        v[rng.random(k) < 0.1] = -3.0
        p2 = rng.random(k) < 0.1
        v[p2] = np.ldexp(1.0, rng.integers(-20, 20, int(p2.sum()))) * rng.choice([-1.0, 1.0], int(p2.sum()))
        return v
    return f


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("zh", ["min", "none", "mix"])
def test_signed_wide_range_columns_match_oracle(dtype, zh):
    """Genes whose values take both signs use the signed bucket map (linear near zero,
    logarithmic beyond); the results must not depend on it."""
    rng = np.random.default_rng(17)
    cols = [(1.0, lambda r: (lambda k: r.standard_normal(k))),
            (0.9, _signed_wide),
            (1.0, lambda r: (lambda k: np.round(r.standard_normal(k) * 40) / 40)),
            (0.6, lambda r: (lambda k: r.standard_normal(k) * 1e-3 + (r.random(k) < 0.01) * 1e4))]
    w = _workload(23, 60_000, cols, 8_000, [300, 900, 2500, 40, 7000, 1200])
    w.data = w.data.astype(dtype)
    assert _oracle_compare(w, zero_handling=zh) == "ok"


def test_bucket_table_size_does_not_change_results():
    """The bucket table (2^9 .. 2^13 entries) only changes the work split: smaller tables mean
    larger buckets and more elements per slab. U1 and P stay the same doubles."""
    from hpdex_gb300.resident import BATCHED, ResidentMatrix
    sizes = [500, 800, 1200, 2000, 3000, 4500, 6000, 700, 650, 5200, 900, 3300]
    w = _workload(3, 150_000, COLUMNS, 30_000, sizes)
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    try:
        plan = M.plan(w.group_id, w.n_targets, zero_handling="min", use_continuity=True)
        plan.run(BATCHED)
        U1a, Pa = plan.download()
        for bits in (12, 10, 9, 13):
            plan.set_bucket_bits(bits)
            plan.run(BATCHED)
            U1b, Pb = plan.download()
            np.testing.assert_array_equal(U1b, U1a)
            np.testing.assert_array_equal(Pb, Pa)
        plan.close()
    finally:
        M.close()


@pytest.mark.parametrize("n_targets", [12, 1200])
def test_run_counter_placement_does_not_change_results(n_targets):
    """The per-warp run counters in shared memory (rounds count repeated groups with them) or in
    global memory (rounds match groups across the warp; big buckets count in global memory) give
    the same doubles, on columns with tie-heavy, dominant-value and impure big buckets; with
    1,200 targets the automatic placement is global memory, and it equals the oracle there."""
    from hpdex_gb300.resident import BATCHED, ResidentMatrix
    rng = np.random.default_rng(17)
    if n_targets == 12:
        sizes = [500, 800, 1200, 2000, 3000, 4500, 6000, 700, 650, 5200, 900, 3300]
        w = _workload(3, 150_000, COLUMNS, 30_000, sizes)
    else:
        sizes = list(rng.integers(20, 90, size=n_targets))
        w = _workload(5, 120_000, COLUMNS, 20_000, sizes)
        assert _oracle_compare(w, zero_handling="min") == "ok"
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    try:
        plan = M.plan(w.group_id, w.n_targets, zero_handling="min", use_continuity=True)
        plan.run(BATCHED)
        U1a, Pa = plan.download()
        for mode in (0, 1, -1):
            plan.set_run_counters(mode)
            plan.run(BATCHED)
            U1b, Pb = plan.download()
            np.testing.assert_array_equal(U1b, U1a)
            np.testing.assert_array_equal(Pb, Pa)
        plan.close()
    finally:
        M.close()
