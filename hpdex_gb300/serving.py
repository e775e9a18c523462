"""Serving loop: DE queries (a grouping over a resident matrix) answered as they arrive.

    srv = Server(workspace_bytes=8 << 30, max_batch=16)
    mid = srv.add_matrix(ResidentMatrix(data, indices, indptr, n_rows))
    q = srv.submit(mid, group_id, n_targets, zero_handling="min", use_continuity=True)
    U1, P = q.result()          # (n_targets, n_genes) float64; q.latency_ms

The C++ worker inside the library admits queries in arrival order against the workspace
budget, coalesces up to `max_batch` of them into one launch of the persistent rank kernel
(one longest-first queue of (query, gene) items) and keeps up to two batches queued on the GPU,
so queries that arrive while others run join the next launch. max_batch=1 gives per-query
launches. `poisson_run` drives a server with a Poisson arrival process and reports p50/p99
latency and throughput.
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from . import _lib
from .resident import ResidentMatrix, make_options


class Query:
    def __init__(self, server: "Server", qid: int, U1: np.ndarray, P: np.ndarray):
        self._server = server
        self.id = qid
        self._U1 = U1
        self._P = P
        self.latency_ms = None
        self._done = False

    def result(self, timeout: float | None = None):
        """Waits for the query; returns (U1, P) or raises the query's error."""
        if not self._done:
            lat = ctypes.c_double()
            st = _lib.lib().hpdex_server_wait(self._server._h, self.id,
                                              -1.0 if timeout is None else float(timeout),
                                              ctypes.byref(lat))
            if st == _lib.HPDEX_ERR_TIMEOUT:
                raise TimeoutError(_lib.lib().hpdex_last_error().decode(errors="replace"))
            self._done = True
            _lib.check(st)
            self.latency_ms = lat.value
        self._U1.flags.writeable = False
        self._P.flags.writeable = False
        return self._U1, self._P


class Server:
    def __init__(self, workspace_bytes: int = 8 << 30, max_batch: int = 16):
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().hpdex_server_create(int(workspace_bytes), int(max_batch),
                                                  ctypes.byref(h)))
        self._h = h
        self._mats = []  # resident matrices stay alive with the server
        self._lock = threading.Lock()

    def add_matrix(self, m: ResidentMatrix) -> int:
        mid = ctypes.c_int32()
        _lib.check(_lib.lib().hpdex_server_add_matrix(self._h, m._h, ctypes.byref(mid)))
        self._mats.append(m)
        return mid.value

    def submit(self, matrix_id: int, group_id, n_targets: int, **options) -> Query:
        m = self._mats[matrix_id]
        gid = np.ascontiguousarray(np.asarray(group_id), dtype=np.int32)
        if gid.size != m.n_rows:
            raise ValueError(f"group_id has {gid.size} entries, the matrix {m.n_rows} rows")
        T = int(n_targets)
        U1 = _lib.result_array((max(T, 0), m.n_cols))
        P = _lib.result_array((max(T, 0), m.n_cols))
        qid = ctypes.c_int64()
        opt = make_options(**options)
        _lib.check(_lib.lib().hpdex_server_submit(self._h, int(matrix_id), gid.ctypes.data, T,
                                                  ctypes.byref(opt), U1.ctypes.data,
                                                  P.ctypes.data, ctypes.byref(qid)))
        return Query(self, qid.value, U1, P)

    def stats(self):
        c, b, ms = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        _lib.check(_lib.lib().hpdex_server_stats(self._h, ctypes.byref(c), ctypes.byref(b),
                                                 ctypes.byref(ms)))
        pr, rk, pv = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _lib.check(_lib.lib().hpdex_server_phase_stats(self._h, ctypes.byref(pr), ctypes.byref(rk),
                                                       ctypes.byref(pv)))
        return {"completed": c.value, "batches": b.value, "busy_ms": ms.value,
                "prep_ms": pr.value, "rank_ms": rk.value, "pvalue_ms": pv.value}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.lib().hpdex_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def random_query(rng, n_rows, ref_range=(1_000, 50_000), targets_range=(1, 200),
                 target_size_range=(20, 5_000)):
    """A grouping as the serving workload draws it: a reference of log-uniform size, 1-200
    targets of log-uniform sizes, cells drawn without replacement, every other cell -1. When
    the draw needs more cells than the matrix has, the sizes shrink proportionally."""
    def logu(lo, hi, size=None):
        return np.exp(rng.uniform(np.log(lo), np.log(hi), size=size))
    ref = int(logu(*ref_range))
    T = int(np.floor(logu(targets_range[0], targets_range[1] + 1)))
    T = max(1, min(T, targets_range[1]))
    sizes = logu(*target_size_range, size=T).astype(np.int64)
    if n_rows < 2 * (T + 1):
        raise ValueError(f"{n_rows} cells cannot hold a reference and {T} targets of 2 cells")
    total = ref + int(sizes.sum())
    if total > n_rows:
        f = n_rows / total
        ref = max(2, int(ref * f))
        sizes = np.maximum(2, (sizes * f).astype(np.int64))
        # every group keeps at least 2 cells (fewer make the query fail "Sample too small")
        while ref + sizes.sum() > n_rows:
            k = int(np.argmax(sizes))
            if sizes[k] > 2:
                sizes[k] -= 1
            else:
                ref -= 1
    perm = rng.permutation(n_rows)
    gid = np.full(n_rows, -1, np.int32)
    gid[perm[:ref]] = 0
    o = ref
    for t, s in enumerate(sizes, start=1):
        gid[perm[o:o + int(s)]] = t
        o += int(s)
    return gid, T


def poisson_run(server: Server, matrix_ids, n_rows_of, rate_qps: float, n_queries: int,
                seed: int = 0, options=None, weights=None):
    """Submits n_queries at Poisson arrival times (rate_qps) over random matrices (chosen with
    `weights`, uniformly by default); waits for all; returns latency percentiles (ms, overall
    and per matrix), throughput (tests/s), and the server's phase times."""
    options = options or dict(zero_handling="min", use_continuity=True, tie_correction=True)
    rng = np.random.default_rng(seed)
    p = None if weights is None else np.asarray(weights, dtype=float) / np.sum(weights)
    plan = []
    for _ in range(n_queries):
        mid = int(rng.choice(matrix_ids, p=p))
        gid, T = random_query(rng, n_rows_of[mid])
        plan.append((mid, gid, T))
    gaps = rng.exponential(1.0 / rate_qps, size=n_queries)
    queries = []
    tests = 0
    t0 = time.perf_counter()
    due = t0
    for (mid, gid, T), gap in zip(plan, gaps):
        due += gap
        while True:
            now = time.perf_counter()
            if now >= due:
                break
            time.sleep(min(due - now, 0.002))
        queries.append(server.submit(mid, gid, T, **options))
        tests += T * server._mats[mid].n_cols
    lat = []
    for q in queries:
        q.result()
        lat.append(q.latency_ms)
    wall = time.perf_counter() - t0
    lat = np.asarray(lat)
    mids = np.asarray([mid for mid, _, _ in plan])
    per_matrix = {}
    for mid in sorted(set(mids.tolist())):
        x = lat[mids == mid]
        per_matrix[int(mid)] = {"queries": int(x.size), "p50_ms": float(np.percentile(x, 50)),
                                "p99_ms": float(np.percentile(x, 99))}
    return {"rate_qps": rate_qps, "queries": n_queries, "tests": tests,
            "tests_per_s": tests / wall, "wall_s": wall,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "per_matrix": per_matrix, **server.stats()}
