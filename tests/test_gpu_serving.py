"""GPU: the serving loop. Every result is the same whether the query runs alone (per-query
launches) or coalesced with others in one launch, and equals the one-shot call; a failing
query reports the reference's error without disturbing the queries batched with it; a budget
smaller than one query still lets each query run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _matrices():
    from hpdex_gb300 import synthetic
    from hpdex_gb300.resident import ResidentMatrix
    a = synthetic.perturb_screen(seed=41, n_rows=20_000, n_cols=300, n_targets=10, ref_size=2_000)
    b = synthetic.umi_counts(seed=42, n_rows=8_000, n_cols=200, n_targets=5)
    return [(a, ResidentMatrix(a.data, a.indices, a.indptr, a.n_rows)),
            (b, ResidentMatrix(b.data, b.indices, b.indptr, b.n_rows))]


def _queries(mats, n, seed):
    from hpdex_gb300.serving import random_query
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        mid = i % len(mats)
        gid, T = random_query(rng, mats[mid][0].n_rows, ref_range=(500, 4_000),
                              targets_range=(1, 12), target_size_range=(20, 800))
        zh = ["min", "max", "mix"][i % 3]
        out.append((mid, gid, T, dict(zero_handling=zh, use_continuity=bool(i % 2),
                                      alternative=["two-sided", "less", "greater"][i % 3])))
    return out


def _run(mats, queries, max_batch, budget=8 << 30):
    from hpdex_gb300.serving import Server
    with Server(workspace_bytes=budget, max_batch=max_batch) as srv:
        ids = [srv.add_matrix(m) for _, m in mats]
        if max_batch == 1:
            res = [srv.submit(ids[mid], gid, T, **o).result() for mid, gid, T, o in queries]
        else:
            qs = [srv.submit(ids[mid], gid, T, **o) for mid, gid, T, o in queries]
            res = [q.result() for q in qs]
        return res, srv.stats()


def test_alone_equals_mixed_equals_oneshot():
    from hpdex_gb300.backend.bin import kernel
    mats = _matrices()
    queries = _queries(mats, 12, seed=5)
    alone, st1 = _run(mats, queries, max_batch=1)
    mixed, st2 = _run(mats, queries, max_batch=16)
    assert st1["batches"] == 12 and st2["batches"] < 12  # the mixed run really coalesced
    for (U1a, Pa), (U1m, Pm) in zip(alone, mixed):
        np.testing.assert_array_equal(U1a, U1m)
        np.testing.assert_array_equal(Pa, Pm)
    zh_code = {"none": 0, "min": 1, "max": 2, "mix": 3}
    alt_code = {"less": 0, "greater": 1, "two-sided": 2}
    for (mid, gid, T, o), (U1, P) in list(zip(queries, alone))[:4]:
        w = mats[mid][0]
        U1o, Po = kernel.mannwhitneyu(w.data, w.indices, w.indptr, gid, T,
                                      use_continuity=o["use_continuity"],
                                      zero_handling=zh_code[o["zero_handling"]],
                                      alternative=alt_code[o["alternative"]], fast_norm=False)
        np.testing.assert_array_equal(U1, U1o)
        np.testing.assert_array_equal(P, Po)


def test_failing_query_does_not_disturb_its_batch():
    from hpdex_gb300.serving import Server
    mats = _matrices()
    w, M = mats[1]
    good = _queries(mats[1:], 3, seed=9)
    bad = np.full(w.n_rows, -1, np.int32)
    bad[:3] = 0   # reference of 3 cells: under zero_handling=none most genes store < 2
    bad[3:6] = 1
    with Server(max_batch=8) as srv:
        mid = srv.add_matrix(M)
        qs = [srv.submit(mid, gid, T, **o) for _, gid, T, o in good[:2]]
        qb = srv.submit(mid, bad, 1, zero_handling="none")
        qs.append(srv.submit(mid, good[2][1], good[2][2], **good[2][3]))
        with pytest.raises(RuntimeError, match="Sample too small"):
            qb.result()
        res = [q.result() for q in qs]
    alone, _ = _run(mats[1:], good, max_batch=1)
    for (U1a, Pa), (U1, P) in zip(alone, res):
        np.testing.assert_array_equal(U1a, U1)
        np.testing.assert_array_equal(Pa, P)


def test_tiny_budget_runs_queries_one_at_a_time():
    mats = _matrices()
    queries = _queries(mats, 4, seed=13)
    res, st = _run(mats, queries, max_batch=16, budget=1)
    assert st["completed"] == 4 and st["batches"] == 4
    ref, _ = _run(mats, queries, max_batch=1)
    for (U1a, Pa), (U1, P) in zip(ref, res):
        np.testing.assert_array_equal(U1a, U1)
        np.testing.assert_array_equal(Pa, P)


def test_phase_stats_account_for_the_device_time():
    """The server's per-phase device times (rank launches, one p-value launch per batch) add up
    to its busy time; host preparation time is reported beside them."""
    from hpdex_gb300.serving import Server
    mats = _matrices()
    queries = _queries(mats, 12, seed=9)
    with Server(workspace_bytes=8 << 30, max_batch=16) as srv:
        ids = [srv.add_matrix(m) for _, m in mats]
        for q in [srv.submit(ids[mid], gid, T, **o) for mid, gid, T, o in queries]:
            q.result()
        st = srv.stats()
    assert st["completed"] == len(queries)
    assert st["rank_ms"] > 0.0 and st["pvalue_ms"] >= 0.0 and st["prep_ms"] > 0.0
    assert abs(st["rank_ms"] + st["pvalue_ms"] - st["busy_ms"]) <= 1e-3 * st["busy_ms"] + 1e-3


def test_matrix_from_device_pointers_equals_host_upload():
    """hpdex_matrix_create_device (values and int32 row ids already in device memory) gives the
    resident matrix the host upload gives: the same plan results, bit for bit."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch sees no CUDA device")
    from hpdex_gb300 import synthetic
    from hpdex_gb300.resident import ResidentMatrix
    w = synthetic.perturb_screen(seed=44, n_rows=12_000, n_cols=200, n_targets=9, ref_size=1_500)
    d = torch.from_numpy(w.data).cuda()
    r = torch.from_numpy(w.indices.astype(np.int32)).cuda()
    torch.cuda.synchronize()
    Md = ResidentMatrix.from_device(d.data_ptr(), r.data_ptr(), w.indptr, w.n_rows, np.float32)
    del d, r
    Mh = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    out = []
    for M in (Md, Mh):
        p = M.plan(w.group_id, w.n_targets, zero_handling="min", use_continuity=True)
        p.run()
        out.append(p.download())
        p.close()
        M.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
