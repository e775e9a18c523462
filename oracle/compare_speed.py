"""Times the oracle port against the reference's own compiled kernel (oracle/_ref, built by
oracle/build_ref.sh) on the CPU-baseline sample of the perturb_screen workload: every 10th
gene of 200,000 cells x 8,000 genes, 500 targets, zero_handling=min, continuity and tie
correction on. Both must agree bit for bit; the script prints their throughput on 1 thread and
on all host threads, and how much of the reference's time its per-group sorts take (the same
call on input whose columns are pre-sorted by value, with ref_sorted / tar_sorted set, so that
the reference skips them).

TEST INFRASTRUCTURE ONLY. Runs where oracle/_ref exists (the machine with the reference
sources):  python oracle/compare_speed.py
"""
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(HERE, "_ref"))
sys.path.insert(0, ROOT)

import kernel as ref  # noqa: E402  (the reference's compiled module)

from hpdex_gb300 import synthetic  # noqa: E402
from oracle import oracle  # noqa: E402


def sample(w, every=10):
    sel = np.arange(0, w.n_cols, every)
    sizes = np.diff(w.indptr)[sel]
    ip = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    idx = np.concatenate([np.arange(w.indptr[c], w.indptr[c + 1]) for c in sel])
    return sel, w.data[idx], w.indices[idx].astype(np.int64), ip


def best(f, reps=3):
    ts = []
    for _ in range(reps):
        t = time.perf_counter()
        f()
        ts.append(time.perf_counter() - t)
    return min(ts), statistics.median(ts)


def main():
    w = synthetic.perturb_screen(seed=7)
    sel, data, ind, ip = sample(w)
    T, gid = w.n_targets, w.group_id
    col = np.repeat(np.arange(ip.size - 1), np.diff(ip))
    o = np.lexsort((data, col))
    sdata, sind = data[o], ind[o]

    def port(th):
        return oracle.mannwhitneyu(data, ind, ip, gid, T, tie_correction=True, use_continuity=True,
                                   zero_handling=1, alternative=2, method=2, threads=th)

    def reference(th, d=data, i=ind, presorted=False):
        return ref.mannwhitneyu(d, i, ip, gid, T, presorted, presorted, True, True, False, 1, 2, 2,
                                th, "csc", False)

    tests = sel.size * T
    print(f"sample: {sel.size} genes x {T} targets = {tests} tests, {data.size} stored values")
    for th in (1, oracle.max_threads()):
        a, b = port(th), reference(th)
        c = reference(th, sdata, sind, True)
        same = (np.array_equal(a[0], np.asarray(b[0])) and np.array_equal(a[1], np.asarray(b[1]))
                and np.array_equal(np.asarray(c[0]), np.asarray(b[0]))
                and np.array_equal(np.asarray(c[1]), np.asarray(b[1])))
        tp, _ = best(lambda: port(th))
        tr, _ = best(lambda: reference(th))
        ts, _ = best(lambda: reference(th, sdata, sind, True))
        print(f"{th:3d} threads: port {tests / tp:.3e} tests/s, reference {tests / tr:.3e} tests/s "
              f"(port/reference {tr / tp:.2f}); reference without its sorts {tests / ts:.3e} "
              f"tests/s (sorts {100 * (tr - ts) / tr:.0f}% of its time); bit-identical: {same}")


if __name__ == "__main__":
    main()
