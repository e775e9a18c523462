"""Benchmark of the MWU differential-expression path on one GB300.

Workload (default): perturbation-screen scale, 200,000 cells x 8,000 genes, log1p-CP10k
float32 (~1.47e8 nonzeros), 20,000 reference cells, 500 targets, zero_handling="min",
tie and continuity corrections, two-sided asymptotic p-values. Synthetic, seeded.

One step = one DE call: per-(gene, target) U1 and P for all 500 x 8,000 tests.
  value : tests/s with the matrix resident in HBM (library layout: float32 values, int32 row
          ids, int64 column pointers, per-column key ranges), batched form (group-id
          preparation + persistent work-queue rank kernel that also computes the p-values,
          replayed as one CUDA graph), device time from CUDA events recorded inside the graph
          on the launching stream. kernels_ms also times the same plan with the p-values in a
          separate kernel.
  e2e   : tests/s through the reference-shaped public call kernel.mannwhitneyu with host
          numpy arrays in and out (H2D of values, int64 row ids, column pointers and
          group ids; D2H of U1 and P), wall clock. The call uploads the matrix in column
          chunks and ranks chunk k while chunk k+1 is in flight; on coherent-memory systems
          the p-value kernel writes U1 and P straight into the output arrays.
  plain : the same plan in the plain form: one single-CTA launch per gene in column order, no
          graph, no queue; the launches go round-robin to up to 128 concurrent streams, so the
          comparison measures the queue and the graph, not idle SMs.
  autotune: the plan's layout tuner (run counters in shared or global memory x bucket table of
          2^13 or 2^12 entries, each candidate timed over 3 batched runs, the fastest kept);
          also on the exact-mode plan, where 1,501 groups make the other choice.
  umi_counts: the 50,000 x 2,000 integer-count workload (49 targets): batched plan with the
          per-gene histogram path against the bucket path only, group means, CPU port.
  exact : the 60,000 x 4,000 dense exact-mode workload (40 reference cells, 1,500 targets):
          both DP variants on the device, the layout tuner, CPU port on a gene sample.
  serving: the serving loop (hpdex_gb300.serving) over five resident matrices (the
          200k x 8k screen, a 50k x 2k log1p-CP10k matrix, a 50k x 2k integer-count matrix,
          and a 1M x 20k log1p-CP10k atlas of 1e9 entries generated on the GPU with its
          integer-count twin; 70 % float / 30 % count queries), Poisson arrivals of random
          groupings (reference 1k-50k cells, 1-200 targets of 20-5,000 cells), p50/p99 latency
          overall and per matrix, tests/s, per-phase device time, coalesced launches
          (max_batch=16) against per-query launches (max_batch=1), at a sustained and a
          saturating arrival rate.
The inputs (1.17 GB resident) exceed the 129 MB L2, so no flush is needed between steps.

--impl reference times the CPU restatement of the reference backend (oracle/, OpenMP over all
host cores) on a bounded sample of genes of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "gene x target MWU tests/s"
UNIT = "tests/s"


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(values, dist):
    """Element-wise maximum of this rank's floats over all ranks (gloo, host side): the job's
    time is its slowest rank's."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_figure(key):
    """A per-launch figure of the rank kernel from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "mwu_rank_kernel_perturb_screen.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def traffic_from_profile():
    """DRAM bytes per rank-kernel launch (dram__bytes_read.sum + dram__bytes_write.sum)."""
    return profile_figure("traffic_bytes_per_launch_full_workload")


class ClockSampler:
    """nvidia-smi clock/throttle sampling (every 50 ms); stop() keeps the samples taken inside
    the timed region (wall-clock window) and says how many there were."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.p = None

    def wait_first(self, timeout=3.0):
        """Returns once nvidia-smi has written a sample (so that sampling covers what follows)."""
        t_end = time.time() + timeout
        while self.p is not None and time.time() < t_end:
            try:
                if os.path.getsize(self.f.name) > 0:
                    return
            except OSError:
                return
            time.sleep(0.01)

    @staticmethod
    def _parse(line):
        import datetime
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 10:
            return None
        try:
            t = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None
        return t, parts[1:]

    def stop(self, t_begin=None, t_end=None):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                r = self._parse(line)
                if r is not None:
                    rows.append(r)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        inside = [r for t, r in rows if t_begin is None or (t_begin <= t <= t_end)]
        if inside:
            use, where = inside, "inside the timed region"
        else:  # a timed region shorter than the sampling period: the sample nearest to it
            mid = 0.5 * (t_begin + t_end)
            use, where = [min(rows, key=lambda tr: abs(tr[0] - mid))[1]], "nearest to the timed region"
        sm = [float(r[1]) for r in use if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in use if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in use for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(use), "where": where}


class NvmlSampler:
    """SM clock and clock-event reasons through NVML's read-only queries, every `period` seconds
    on a host thread, so that even a timed region of tens of milliseconds holds many samples.
    stop() keeps the samples inside the timed region. Raises OSError when NVML is unavailable
    (ClockSampler, over nvidia-smi, is the fallback)."""

    # nvmlClocksEventReason bits (nvml.h)
    BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
            0x40: "hw_thermal_slowdown"}

    def __init__(self, gpu_index=0, period=0.002):
        import ctypes
        import threading
        self.ct = ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.lib = lib
        self.h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(gpu_index), ctypes.byref(self.h)) != 0:
            raise OSError("no NVML device")
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        lib.nvmlDeviceGetMaxClockInfo(self.h, ctypes.c_int(1), ctypes.byref(mx))  # NVML_CLOCK_SM
        self.max_mhz = float(mx.value)
        self.rows = []
        self.period = period
        self.done = threading.Event()
        self.t = threading.Thread(target=self._loop, daemon=True)
        self.t.start()

    def _loop(self):
        ct = self.ct
        c, r = ct.c_uint(), ct.c_ulonglong()
        while not self.done.is_set():
            t = time.time()
            if self.lib.nvmlDeviceGetClockInfo(self.h, ct.c_int(1), ct.byref(c)) == 0 and \
                    self.reasons_fn(self.h, ct.byref(r)) == 0:
                self.rows.append((t, float(c.value), int(r.value)))
            time.sleep(self.period)

    def wait_first(self, timeout=3.0):
        t_end = time.time() + timeout
        while not self.rows and time.time() < t_end:
            time.sleep(0.001)

    def stop(self, t_begin=None, t_end=None):
        self.done.set()
        self.t.join(timeout=2)
        rows = self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["no samples"]}
        inside = [x for x in rows if t_begin is None or t_begin <= x[0] <= t_end]
        where = "inside the timed region"
        if not inside:
            mid = 0.5 * (t_begin + t_end)
            inside, where = [min(rows, key=lambda x: abs(x[0] - mid))], "nearest to the timed region"
        reasons = sorted({name for x in inside for bit, name in self.BITS.items() if x[2] & bit})
        return {"sm_mhz": statistics.median(x[1] for x in inside), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(inside), "where": where,
                "source": f"NVML every {self.period * 1e3:.0f} ms"}


def clock_sampler():
    try:
        return NvmlSampler(0)
    except (OSError, AttributeError):
        return ClockSampler(0)


def make_workload(args, rank):
    from hpdex_gb300 import synthetic
    return synthetic.perturb_screen(seed=7 + rank)


def algorithmic_bytes(w):
    """Compulsory DRAM bytes of one rank-kernel launch: float32 value + int32 row id per
    nonzero, the column pointers, the group ids, and U1 + tie sum (8 B each) per test."""
    C, T = w.n_cols, w.n_targets
    return w.nnz * 8 + 8 * (C + 1) + 4 * w.n_rows + 16 * C * T


def cpu_sample(w, max_genes):
    """Every k-th gene, so the sample keeps the gene-size distribution."""
    k = max(1, w.n_cols // max_genes)
    sel = np.arange(0, w.n_cols, k)
    sizes = np.diff(w.indptr)[sel]
    ip = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    idx = np.concatenate([np.arange(w.indptr[c], w.indptr[c + 1]) for c in sel])
    return sel, w.data[idx], w.indices[idx], ip


def time_cpu(w, max_genes, reps=1):
    from oracle import oracle
    sel, data, ind, ip = cpu_sample(w, max_genes)
    best = None
    for _ in range(reps):
        t = time.perf_counter()
        oracle.mannwhitneyu(data, ind, ip, w.group_id, w.n_targets, tie_correction=True,
                            use_continuity=True, zero_handling=1, alternative=2, method=2,
                            threads=-1)
        dt = time.perf_counter() - t
        best = dt if best is None else min(best, dt)
    tests = sel.size * w.n_targets
    return tests / best, oracle.max_threads(), f"{sel.size} of {w.n_cols} genes (every {w.n_cols // sel.size}th), all 500 targets, {tests} tests, best of {reps}"


def host_cpu():
    """The host CPU's model name as lscpu reports it (Arm hosts have no 'model name' line in
    /proc/cpuinfo), with the logical CPU count."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() == "Model name":
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return f"{model or platform.machine()}, {os.cpu_count()} logical CPUs"


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    w = make_workload(args, 0)
    for _ in range(args.warmup):
        time_cpu(w, 100)
    vals = []
    cores = None
    sample = None
    for _ in range(args.steps):
        v, cores, sample = time_cpu(w, args.cpu_genes)
        vals.append(v)
    value = statistics.median(vals)
    tests_per_step = cpu_sample(w, args.cpu_genes)[0].size * w.n_targets
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        # a step is one bounded sample of the workload (config.sample), timed on the host
        "ms_per_step": tests_per_step / value * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "perturb_screen 200000 cells x 8000 genes x 500 targets, "
                               "log1p-CP10k float32, zero_handling=min", "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample, "cpu": host_cpu()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def serving_leg(M, w, queries=120, rates=(40.0, 2000.0)):
    """Serving loop over five resident matrices (see module doc): the screen, a 50k x 2k
    log1p-CP10k matrix, an integer-count 50k x 2k matrix, and the 1M x 20k atlas
    (1e9 entries, generated on the GPU) with its integer-count twin. 70 % of the queries go to
    the float matrices, 30 % to the integer-count ones. Arrivals are Poisson at a sustained
    rate and at a saturating one, with coalesced (max_batch 16) and per-query launches."""
    from hpdex_gb300 import synthetic
    from hpdex_gb300.resident import ResidentMatrix
    from hpdex_gb300.serving import Server, poisson_run
    b = synthetic.perturb_screen(seed=3, n_rows=50_000, n_cols=2_000, n_targets=50, ref_size=5_000)
    c = synthetic.umi_counts(seed=4, n_rows=50_000, n_cols=2_000)
    t_gen = time.perf_counter()
    atlas, atlas_counts = synthetic.resident_atlas()
    t_gen = time.perf_counter() - t_gen
    mats = [M, ResidentMatrix(b.data, b.indices, b.indptr, b.n_rows),
            ResidentMatrix(c.data, c.indices, c.indptr, c.n_rows), atlas, atlas_counts]
    names = ["screen 200000x8000 float", "50000x2000 float", "50000x2000 counts",
             "atlas 1000000x20000 float", "atlas 1000000x20000 counts"]
    rows = {0: w.n_rows, 1: b.n_rows, 2: c.n_rows, 3: atlas.n_rows, 4: atlas_counts.n_rows}
    weights = [0.7 / 3, 0.7 / 3, 0.3 / 2, 0.7 / 3, 0.3 / 2]
    runs = []
    for mode, mb in (("coalesced", 16), ("per_query", 1)):
        for rate in rates:
            with Server(workspace_bytes=64 << 30, max_batch=mb) as srv:
                ids = [srv.add_matrix(m) for m in mats]
                poisson_run(srv, ids, rows, rate_qps=rate, n_queries=10, seed=1, weights=weights)
                base = srv.stats()
                r = poisson_run(srv, ids, rows, rate_qps=rate, n_queries=queries, seed=2,
                                weights=weights)
            runs.append({"mode": mode, "max_batch": mb, "rate_qps": rate,
                         "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"], "mean_ms": r["mean_ms"],
                         "tests_per_s": r["tests_per_s"], "launches": r["batches"] - base["batches"],
                         "gpu_busy_ms": r["busy_ms"] - base["busy_ms"],
                         "phase_ms": {"host_prep": r["prep_ms"] - base["prep_ms"],
                                      "rank": r["rank_ms"] - base["rank_ms"],
                                      "pvalue": r["pvalue_ms"] - base["pvalue_ms"]},
                         "per_matrix": {names[k]: v for k, v in r["per_matrix"].items()}})
    # small queries only (the two 50k x 2k matrices), where one launch per query leaves SMs
    # idle and coalescing several queries into one launch can pay
    small = []
    for mode, mb in (("coalesced", 16), ("per_query", 1)):
        with Server(workspace_bytes=64 << 30, max_batch=mb) as srv:
            ids = [srv.add_matrix(m) for m in mats[1:3]]
            srows = {ids[0]: b.n_rows, ids[1]: c.n_rows}
            poisson_run(srv, ids, srows, rate_qps=5000.0, n_queries=20, seed=3, weights=[0.7, 0.3])
            base = srv.stats()
            r = poisson_run(srv, ids, srows, rate_qps=5000.0, n_queries=400, seed=4, weights=[0.7, 0.3])
        small.append({"mode": mode, "max_batch": mb, "rate_qps": 5000.0, "p50_ms": r["p50_ms"],
                      "p99_ms": r["p99_ms"], "tests_per_s": r["tests_per_s"],
                      "launches": r["batches"] - base["batches"],
                      "phase_ms": {"host_prep": r["prep_ms"] - base["prep_ms"],
                                   "rank": r["rank_ms"] - base["rank_ms"],
                                   "pvalue": r["pvalue_ms"] - base["pvalue_ms"]}})
    atlas.close()
    atlas_counts.close()
    return {"matrices": names, "atlas_nnz": 1_000_000_000, "atlas_generation_s": t_gen,
            "small_queries_saturated": small,
            "query_mix": "70 % float / 30 % integer counts", "queries_per_run": queries,
            "arrival": "Poisson", "rates": {"sustained_qps": rates[0], "saturating_qps": rates[1]},
            "runs": runs,
            "note": "latency = submit to results in host memory; tests/s over the run's wall time; "
                    "phase_ms = host preparation of the batches, device time of the rank and "
                    "p-value launches (one p-value launch per batch)"}


def time_plan(plan, steps, warmup=2):
    """Device times (ms, CUDA events of the plan's stream) of `steps` batched runs."""
    from hpdex_gb300.resident import BATCHED
    for _ in range(warmup):
        plan.run(BATCHED)
    tot, rk = [], []
    for _ in range(steps):
        plan.run(BATCHED)
        (t, r, _), _ = plan.timings()
        tot.append(t)
        rk.append(r)
    return statistics.mean(tot), statistics.mean(rk)


def time_cpu_workload(w, max_genes, reps, **opt):
    """The oracle port (OpenMP, all host cores) on every k-th gene of w: tests/s, best of reps."""
    from oracle import oracle
    sel, data, ind, ip = cpu_sample(w, max_genes)
    best = None
    for _ in range(reps):
        t = time.perf_counter()
        oracle.mannwhitneyu(data, ind, ip, w.group_id, w.n_targets, threads=-1, **opt)
        dt = time.perf_counter() - t
        best = dt if best is None else min(best, dt)
    tests = sel.size * w.n_targets
    return tests / best, oracle.max_threads(), \
        f"{sel.size} of {w.n_cols} genes, all {w.n_targets} targets, {tests} tests, best of {reps}"


def umi_leg(hbm, steps=20):
    """Integer-count workload (50,000 cells x 2,000 genes, NB counts, 10,000 reference cells,
    49 targets, zero_handling=min): the batched plan with the per-gene histogram path against the
    same plan on the bucket path only; group means over G = 50; the oracle port on the host."""
    from hpdex_gb300 import synthetic
    from hpdex_gb300.resident import ResidentMatrix
    w = synthetic.umi_counts()
    T, C = w.n_targets, w.n_cols
    tests = T * C
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    plan = M.plan(w.group_id, T, zero_handling="min", use_continuity=True, tie_correction=True)
    hist_tot, hist_rank = time_plan(plan, steps)
    U1h, Ph = plan.download()
    plan.set_histogram(False)
    buck_tot, buck_rank = time_plan(plan, steps)
    U1b, Pb = plan.download()
    plan.close()
    gm = []
    for _ in range(4):
        t = time.perf_counter()
        M.group_mean(w.group_id, T + 1, include_zeros=True)
        gm.append(time.perf_counter() - t)
    M.close()
    B = algorithmic_bytes(w)
    cpu_v, cores, sample = time_cpu_workload(w, C, 3, tie_correction=True, use_continuity=True,
                                             zero_handling=1, alternative=2, method=2)
    return {"workload": f"umi_counts: 50000 cells x 2000 genes, integral float32 NB counts "
                        f"(realised density {w.nnz / (w.n_rows * C):.3f}, nnz={w.nnz}), 10000 "
                        f"reference cells, {T} targets, zero_handling=min, tie+continuity",
            "histogram": {"value": tests / (hist_tot / 1e3), "unit": UNIT, "ms_per_step": hist_tot,
                          "rank_ms": hist_rank,
                          "roofline": {"achieved": B / (hist_rank / 1e3) / 1e9, "peak": hbm,
                                       "unit": "GB/s", "frac": B / (hist_rank / 1e3) / 1e9 / hbm,
                                       "algorithmic_bytes": B}},
            "bucket_only": {"value": tests / (buck_tot / 1e3), "unit": UNIT,
                            "ms_per_step": buck_tot, "rank_ms": buck_rank},
            "histogram_speedup": buck_tot / hist_tot,
            "results_identical": bool(np.array_equal(U1h, U1b) and np.array_equal(Ph, Pb)),
            "group_mean_ms": {"median": statistics.median(gm) * 1e3, "groups": T + 1,
                              "note": "hpdex_matrix_group_mean, include_zeros, host wall incl. D2H"},
            "steps": steps,
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample}}


def exact_leg(steps=3):
    """Exact-mode workload (60,000 cells x 4,000 genes dense float32 N(0,1) with per-target
    shifts, 40 reference cells, 1,500 targets of 3-40 cells, zero_handling=none): device tests/s
    for the reference-compatible DP variant and the true-null variant (rank kernel, then the
    table build and lookup), and the oracle port on a gene sample on the host."""
    from hpdex_gb300 import synthetic
    from hpdex_gb300.resident import ResidentMatrix
    w = synthetic.exact_small()
    T, C = w.n_targets, w.n_cols
    tests = T * C
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    out = {"workload": "exact_small: 60000 cells x 4000 genes dense float32 (nnz 2.4e8), 40 "
                       f"reference cells, {T} targets of 3-40 cells, zero_handling=none, "
                       "method=exact, tie correction on, no continuity"}
    for variant in ("reference", "mwu_null"):
        plan = M.plan(w.group_id, T, zero_handling="none", use_continuity=False,
                      tie_correction=True, method="exact", exact_variant=variant)
        from hpdex_gb300.resident import BATCHED
        plan.run(BATCHED)
        tt, rk, tb = [], [], []
        for _ in range(steps):
            plan.run(BATCHED)
            (t, r, p), _ = plan.timings()
            tt.append(t)
            rk.append(r)
            tb.append(p)
        if variant == "reference":  # the layout tuner on this plan (1,501 groups)
            out["autotune"] = plan.autotune(reps=3)
        plan.close()
        out[variant] = {"value": tests / (statistics.median(tt) / 1e3), "unit": UNIT,
                        "ms_per_step": statistics.median(tt), "rank_ms": statistics.median(rk),
                        "tables_and_lookup_ms": statistics.median(tb)}
    M.close()
    cpu_v, cores, sample = time_cpu_workload(w, 200, 1, tie_correction=True, use_continuity=False,
                                             zero_handling=0, alternative=2, method=1)
    out["cpu_baseline"] = {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port",
                           "variant": "reference (the reference's uint64 DP)", "sample": sample,
                           "full_workload_s_estimate": tests / cpu_v}
    out["reference_note"] = ("the reference's p_exact / p_exact_parallel "
                             "(src/cpp/mannwhitneyu.cpp:98-188, :243-282); a survey-container "
                             "estimate for the whole workload is about 15.3 s on 8 x86 cores")
    return out


def run_ours(args, rank, world):
    from hpdex_gb300 import _lib
    from hpdex_gb300.backend.bin import kernel
    from hpdex_gb300.resident import BATCHED, PLAIN, ResidentMatrix

    if _lib.device_count() < 1:
        raise RuntimeError("no CUDA device")
    w = make_workload(args, rank)
    T, C = w.n_targets, w.n_cols
    tests = T * C
    if args.only_oneshot:  # profiling runs: the public call only (warm-up, then `steps` calls)
        kw = dict(tie_correction=True, use_continuity=True, zero_handling=1, fast_norm=False)
        for _ in range(max(1, args.warmup)):
            kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, T, **kw)
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, T, **kw)
            ts.append(time.perf_counter() - t0)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unit": UNIT, "form": "one-shot public call",
                              "value": tests / statistics.median(ts),
                              "median_ms": statistics.median(ts) * 1e3}), flush=True)
        return 0
    if args.only_batched and args.workload != "screen":
        # profiling runs on the other workloads: the batched plan only
        from hpdex_gb300 import synthetic
        w = synthetic.umi_counts() if args.workload == "umi" else synthetic.exact_small()
        T, C = w.n_targets, w.n_cols
        tests = T * C
        opt = (dict(zero_handling="min", use_continuity=True, tie_correction=True)
               if args.workload == "umi" else
               dict(zero_handling="none", use_continuity=False, tie_correction=True, method="exact"))
    else:
        opt = dict(zero_handling="min", use_continuity=True, tie_correction=True)
    M = ResidentMatrix(w.data, w.indices, w.indptr, w.n_rows)
    plan = M.plan(w.group_id, T, **opt)
    if args.only_batched and args.separate_pvalues:
        plan.set_fused_pvalues(False)
    sampler = clock_sampler()  # sampling from before the warm-up on
    for _ in range(max(3, args.warmup)):
        plan.run(BATCHED)
    U1, P = plan.download()

    dist = None
    if world > 1:
        import torch.distributed as dist  # host-side barrier / max only
        dist.init_process_group("gloo")
        dist.barrier()
    sampler.wait_first()
    tw0 = time.time()
    t0 = time.perf_counter()
    dev_ms, rank_ms, p_ms, launches = [], [], [], 0
    for _ in range(args.steps):
        plan.run(BATCHED)  # synchronous: graph replay + sync + error check
        (tot, rk, pv), nl = plan.timings()
        dev_ms.append(tot)
        rank_ms.append(rk)
        p_ms.append(pv)
        launches += nl
    wall = time.perf_counter() - t0
    clocks = sampler.stop(tw0, time.time())
    elapsed_dev = sum(dev_ms) / 1e3
    if dist is not None:
        elapsed_dev, wall = max_over_ranks([elapsed_dev, wall], dist)
    value = world * tests * args.steps / elapsed_dev

    line_core = {"value": value, "ms_per_step": statistics.mean(dev_ms),
                 "rank_ms": statistics.mean(rank_ms), "pvalue_ms": statistics.mean(p_ms)}
    if args.only_batched:  # profiling runs: the timed batched steps only
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unit": UNIT, "form": "batched", **line_core}),
                  flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # the same plan with the p-values in a separate kernel after the rank kernel (context for
    # the fused stage's gain; not timed as the metric)
    plan.set_fused_pvalues(False)
    sep = []
    for _ in range(3):
        plan.run(BATCHED)
        sep.append(plan.timings()[0])
    U1s, Ps = plan.download()
    plan.set_fused_pvalues(True)
    same_sep = bool(np.array_equal(U1s, U1) and np.array_equal(Ps, P))

    # plain form (one launch per gene, no graph, no queue), one step
    t1 = time.perf_counter()
    plan.run(PLAIN)
    (ptot, prk, ppv), pl = plan.timings()
    plain_wall = time.perf_counter() - t1
    U1p, Pp = plan.download()
    same = bool(np.array_equal(U1p, U1) and np.array_equal(Pp, P))

    # the layout tuner on the same plan: each candidate layout timed, the fastest kept
    tuned = plan.autotune(reps=3)
    U1t, Pt = plan.download()
    tuned["results_identical"] = bool(np.array_equal(U1t, U1) and np.array_equal(Pt, P))

    # end to end through the public call: host arrays in, host arrays out
    h2d = w.nnz * (w.data.itemsize + 8) + 8 * (C + 1) + 4 * w.n_rows
    d2h = 2 * 8 * tests
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, T, tie_correction=True,
                        use_continuity=True, zero_handling=1, fast_norm=False)  # warm-up
    e2e_calls = []
    for _ in range(e2e_steps):
        te = time.perf_counter()
        U1e, Pe = kernel.mannwhitneyu(w.data, w.indices, w.indptr, w.group_id, T,
                                      tie_correction=True, use_continuity=True, zero_handling=1,
                                      fast_norm=False)
        e2e_calls.append(time.perf_counter() - te)
    e2e_wall = sum(e2e_calls) / e2e_steps
    same = same and bool(np.array_equal(U1e, U1) and np.array_equal(Pe, P))
    # the same call with int32 row ids (scipy's index type), which go to the device as they are
    idx32 = w.indices.astype(np.int32)
    kernel.mannwhitneyu(w.data, idx32, w.indptr, w.group_id, T, tie_correction=True,
                        use_continuity=True, zero_handling=1, fast_norm=False)  # warm-up
    e2e32 = []
    for _ in range(e2e_steps):
        te = time.perf_counter()
        U1i, Pi = kernel.mannwhitneyu(w.data, idx32, w.indptr, w.group_id, T, tie_correction=True,
                                      use_continuity=True, zero_handling=1, fast_norm=False)
        e2e32.append(time.perf_counter() - te)
    same32 = bool(np.array_equal(U1i, U1) and np.array_equal(Pi, P))
    h2d32 = w.nnz * (w.data.itemsize + 4) + 8 * (C + 1) + 4 * w.n_rows

    serving = serving_leg(M, w) if not args.no_serving else None
    hbm, peak_kind = peaks()
    umi = umi_leg(hbm) if not args.no_extra else None
    exact = exact_leg() if not args.no_extra else None

    B = algorithmic_bytes(w)
    rank_avg = statistics.mean(rank_ms) / 1e3
    achieved = B / rank_avg / 1e9
    traffic = traffic_from_profile()
    # the kernel is issue-bound: warp instructions per launch (ncu smsp__inst_executed.sum)
    # over the event time, against 4 issue slots per SM per cycle at the sampled SM clock
    inst = profile_figure("warp_instructions_per_launch_full_workload")
    issue = None
    if inst and clocks.get("sm_mhz"):
        import ctypes
        from hpdex_gb300 import _lib
        sms = ctypes.c_int32()
        _lib.check(_lib.lib().hpdex_device_sm_count(ctypes.byref(sms)))
        issue_peak = 4 * sms.value * clocks["sm_mhz"] * 1e6
        issue = {"achieved": inst / rank_avg, "peak": issue_peak, "unit": "warp inst/s",
                 "frac": inst / rank_avg / issue_peak,
                 "note": "ncu smsp__inst_executed.sum per launch / event time; "
                         "peak = 4 sub-partitions x SMs x sampled SM clock"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": statistics.mean(dev_ms),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32 keys / i64 rank sums / f64 p", "data": "synthetic",
        "config": {"workload": "perturb_screen: 200000 cells x 8000 genes, log1p-CP10k float32, "
                               f"nnz={w.nnz}, 20000 reference cells, {T} targets, "
                               "zero_handling=min, tie+continuity, two-sided asymptotic",
                   "form": "batched (persistent work-queue kernel + CUDA graph)",
                   "l2": "inputs 1.17 GB resident > 129 MB L2 (no flush needed)",
                   "wall_ms_per_step": wall / args.steps * 1e3},
        # median over the calls, as the reference arm reports the median over its steps; the
        # mean (which a call stalled by the shared host can move by tens of ms) is beside it
        "e2e": {"value": world * tests / statistics.median(e2e_calls), "unit": UNIT,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": statistics.median(e2e_calls) * 1e3, "aggregate": "median",
                "calls": e2e_steps, "mean_ms": e2e_wall * 1e3,
                "value_from_mean": world * tests / e2e_wall,
                "min_ms": min(e2e_calls) * 1e3, "max_ms": max(e2e_calls) * 1e3,
                "note": f"median {statistics.median(e2e_calls) * 1e3:.2f} ms, mean "
                        f"{e2e_wall * 1e3:.2f} ms over {e2e_steps} calls",
                "call": "hpdex_gb300.backend.bin.kernel.mannwhitneyu (host numpy in/out, "
                        "fast_norm=False as the reference wrapper passes it)",
                "int32_row_ids": {"value": world * tests / statistics.median(e2e32), "unit": UNIT,
                                  "ms_per_step": statistics.median(e2e32) * 1e3,
                                  "mean_ms": sum(e2e32) / e2e_steps * 1e3,
                                  "h2d_bytes_per_step": int(h2d32), "results_identical": same32,
                                  "note": "the same call with int32 row ids, uploaded as they are"}},
        "plain": {"value": tests / (ptot / 1e3), "unit": UNIT, "ms_per_step": ptot,
                  "wall_ms": plain_wall * 1e3, "launches": pl,
                  "batched_speedup": (tests / elapsed_dev * args.steps) / (tests / (ptot / 1e3)),
                  "results_identical": same},
        "autotune": tuned,
        "kernels_ms": {"rank_with_fused_pvalues": statistics.mean(rank_ms),
                       "separate_form": {"rank": min(x[1] for x in sep),
                                         "pvalue": min(x[2] for x in sep),
                                         "total": min(x[0] for x in sep),
                                         "results_identical": same_sep}},
        "serving": serving,
        "umi_counts": umi,
        "exact": exact,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "kernel": "mwu_rank_kernel", "algorithmic_bytes": B,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "issue": issue},
        "clocks": clocks,
        "gpu_launches": launches,
    }
    if rank == 0:
        cpu_v, cores, sample = time_cpu(w, args.cpu_genes, reps=3)  # best of 3
        line["cpu_baseline"] = {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": sample, "cpu": host_cpu()}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 300 for ours: about 1 s, so that the 50 ms clock "
                         "samples fall inside the timed region; 3 for --impl reference)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-genes", type=int, default=800)
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop leg")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the integer-count and exact-mode legs")
    ap.add_argument("--only-batched", action="store_true",
                    help="time the batched form only (no plain form, e2e or CPU legs); for ncu")
    ap.add_argument("--only-oneshot", action="store_true",
                    help="time the public one-shot call only (for ncu)")
    ap.add_argument("--separate-pvalues", action="store_true",
                    help="with --only-batched: p-values in a separate kernel (for ncu)")
    ap.add_argument("--workload", choices=["screen", "umi", "exact"], default="screen",
                    help="with --only-batched: the 200k x 8k screen (default), the 50k x 2k "
                         "integer-count workload or the 60k x 4k exact-mode workload (for ncu)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 3 if args.impl == "reference" else 300
    rank, world, local = dist_env()
    if world > 1:
        # one process per GPU: each rank sees only its own device (independent replicas)
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
