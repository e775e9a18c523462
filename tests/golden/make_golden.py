"""Generates the golden fixtures in tests/golden/ from the reference's own CPU kernel.

Run in a checkout that has the reference sources (AI4Cell/hpdex) at /root/reference or
$HPDEX_REFERENCE_ROOT:
    oracle/build_ref.sh && python tests/golden/make_golden.py
(`python tests/golden/make_golden.py extreme_shift` writes the deep-tail fixture alone.)
The reference module `kernel` (src/cpp/module.cpp) is built from its unmodified sources by
oracle/build_ref.sh into oracle/_ref/. Every fixture stores its inputs next to the
reference's outputs, so the tests never need the reference at run time.

Reference binding quirk recorded in the fixtures: kernel.group_mean forwards `threads` into
the `use_kahan` parameter and `use_kahan` into `threads` (module.cpp:211-213 versus the
signature at :111-120). Kahan summation is therefore on whenever threads != 0; the
fixtures record both summation modes (threads=0 -> plain, threads=1 -> Kahan).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, ROOT)

import kernel as ref  # noqa: E402  (the reference's compiled module)

from hpdex_gb300 import synthetic  # noqa: E402


def run_ref(data, indices, indptr, gid, T, o):
    try:
        U1, P = ref.mannwhitneyu(data, indices.astype(np.int64), indptr.astype(np.int64), gid, T,
                                 False, False, o["tie_correction"], o["use_continuity"], False,
                                 o["zero_handling"], o["alternative"], o["method"], 1, "csc", False)
        return np.asarray(U1), np.asarray(P), ""
    except RuntimeError as e:
        return np.zeros(0), np.zeros(0), str(e)


def run_means(data, indices, indptr, gid, G, include_zeros):
    plain = ref.group_mean(data, indices.astype(np.int64), indptr.astype(np.int64), gid, G,
                           include_zeros, 0, False, "csc")
    kahan = ref.group_mean(data, indices.astype(np.int64), indptr.astype(np.int64), gid, G,
                           include_zeros, 1, False, "csc")
    return np.asarray(plain), np.asarray(kahan)


def save(name, data, indices, indptr, gid, T, o, n_rows=None):
    U1, P, err = run_ref(data, indices, indptr, gid, T, o)
    G = T + 1
    mp, mk = run_means(data, indices, indptr, gid, G, True)
    mpx, mkx = run_means(data, indices, indptr, gid, G, False)
    idx_dtype = np.int32 if (indices.size == 0 or (indices.max() < 2**31 and indices.min() >= -2**31)) else np.int64
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        data=data, indices=indices.astype(idx_dtype), indptr=indptr.astype(np.int64),
        group_id=gid.astype(np.int32), n_targets=np.int64(T), options=json.dumps(o),
        U1=U1, P=P, error=err, mean_plain=mp, mean_kahan=mk, mean_plain_nz=mpx,
        mean_kahan_nz=mkx)
    return err


def random_case(rng, R, C, T, dtype, dens, neg, ties, nonfinite, bad_rows=False, big_ints=False):
    X = rng.standard_normal((R, C))
    if ties:
        X = np.round(X * 2.0)
    if not neg:
        X = np.abs(X)
    X[rng.random((R, C)) > dens] = 0.0
    if np.issubdtype(dtype, np.integer):
        X = np.round(X * 3.0)
        if np.issubdtype(dtype, np.unsignedinteger):
            X = np.abs(X)
        info = np.iinfo(dtype)
        X = np.clip(X, info.min, info.max)
    X = X.astype(dtype)
    if big_ints:
        base = np.array(2**60, dtype=dtype)
        nz = X != 0
        X[nz] = base + X[nz].astype(dtype)  # values above 2**53 collapse when cast to double
    if nonfinite and np.issubdtype(dtype, np.floating):
        X[rng.random((R, C)) < 0.05] = np.nan
        X[rng.random((R, C)) < 0.03] = np.inf
        X[rng.random((R, C)) < 0.03] = -np.inf
    # CSC with explicit storage of every nonzero (and of the non-finite values)
    rows, cols = np.nonzero((X != 0) | ~np.isfinite(X.astype(np.float64)))
    order = np.lexsort((rows, cols))
    rows, cols = rows[order], cols[order]
    data = X[rows, cols]
    indptr = np.zeros(C + 1, np.int64)
    np.add.at(indptr, cols + 1, 1)
    indptr = np.cumsum(indptr)
    indices = rows.astype(np.int64)
    if bad_rows and indices.size > 4:
        k = rng.choice(indices.size, size=3, replace=False)
        indices[k[0]] = R + 5       # out of range: the reference skips it
        indices[k[1]] = -3          # negative: skipped too
    gid = rng.integers(-1, T + 2, R).astype(np.int32)  # includes -1 and T+1 (both ignored)
    gid[:4] = 0
    for t in range(1, T + 1):
        gid[4 + 2 * (t - 1): 4 + 2 * t] = t
    return data, indices, indptr, gid


def input_digest(w):
    """sha256 over the workload's arrays, stored beside its outputs so that a generator that
    no longer reproduces the inputs fails loudly instead of comparing against stale outputs."""
    import hashlib
    h = hashlib.sha256()
    for a in (w.data, w.indices.astype(np.int64), w.indptr.astype(np.int64),
              w.group_id.astype(np.int32)):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def extreme_shift():
    """Deep-tail fixture: the reference's U1 and P on synthetic.extreme_shift() (20,000
    reference cells against targets of 3,000 / 1,000 / 3,000 cells, |z| up to ~90), for all
    three alternatives with zero_handling='min' and both corrections on. Only the outputs and
    an input digest are stored: the inputs regenerate from the seed (integer draws only)."""
    w = synthetic.extreme_shift()
    out = {}
    for alt in (0, 1, 2):
        o = dict(tie_correction=True, use_continuity=True, zero_handling=1, alternative=alt,
                 method=2)
        U1, P, err = run_ref(w.data, w.indices, w.indptr, w.group_id, w.n_targets, o)
        assert not err, err
        out[f"U1_alt{alt}"] = U1
        out[f"P_alt{alt}"] = P
    np.savez_compressed(os.path.join(HERE, "extreme_shift_outputs.npz"),
                        digest=input_digest(w), n_targets=np.int64(w.n_targets), **out)
    return "extreme_shift_outputs"


def main():
    if sys.argv[1:] == ["extreme_shift"]:
        print("wrote", extreme_shift())
        return
    written = []
    # 1) the CPU-runnable workload: 2,000 cells x 500 genes, 4 targets, min / tie / continuity
    w = synthetic.small_float()
    o = dict(tie_correction=True, use_continuity=True, zero_handling=1, alternative=2, method=2)
    save("small_float", w.data, w.indices, w.indptr, w.group_id, w.n_targets, o)
    written.append("small_float")

    # 2) option and dtype sweep on small random matrices
    rng = np.random.default_rng(20240601)
    dtypes = [np.float32, np.float64, np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32,
              np.int64, np.uint64]
    k = 0
    for zh in range(4):
        for alt in range(3):
            for method in (2, 1):
                for tie in (True, False):
                    dtype = dtypes[k % len(dtypes)]
                    k += 1
                    R = 36 if method == 1 else int(rng.integers(40, 160))
                    C = int(rng.integers(3, 12))
                    T = int(rng.integers(1, 5))
                    data, indices, indptr, gid = random_case(
                        rng, R, C, T, dtype,
                        dens=float(rng.uniform(0.85, 1.0) if zh == 0 else rng.uniform(0.3, 0.95)),
                        neg=(k % 2 == 0),
                        ties=(k % 3 != 0), nonfinite=(k % 4 == 0), bad_rows=(k % 5 == 0))
                    o = dict(tie_correction=tie, use_continuity=bool(k % 2), zero_handling=zh,
                             alternative=alt, method=method)
                    name = f"sweep_{k:03d}"
                    save(name, data, indices, indptr, gid, T, o)
                    written.append(name)

    # 3) edge cases
    o_min = dict(tie_correction=True, use_continuity=True, zero_handling=1, alternative=2, method=2)
    # 3a) 64-bit integers above 2**53 that collapse to equal doubles
    for dt in (np.int64, np.uint64):
        data, indices, indptr, gid = random_case(rng, 80, 6, 2, dt, 0.8, False, True, False,
                                                 big_ints=True)
        save(f"edge_bigint_{np.dtype(dt).name}", data, indices, indptr, gid, 2, o_min)
        written.append(f"edge_bigint_{np.dtype(dt).name}")
    # 3b) empty columns and an all-empty matrix part, plus columns with one entry
    R, C = 50, 6
    gid = np.array([0] * 20 + [1] * 15 + [2] * 15, np.int32)
    indptr = np.array([0, 0, 1, 1, 5, 5, 9], np.int64)
    indices = np.array([3, 0, 21, 36, 49, 1, 2, 30, 31], np.int64)
    data = np.array([1.5, -2.0, 0.0, 3.0, 1.5, 2.0, 2.0, 2.0, -0.0], np.float32)
    for zh in range(1, 4):
        o = dict(o_min, zero_handling=zh)
        save(f"edge_sparse_cols_zh{zh}", data, indices, indptr, gid, 2, o)
        written.append(f"edge_sparse_cols_zh{zh}")
    # 3c) error paths: reference too small, a target too small, per-column errors in 'none'
    gid_small_ref = np.array([0] + [1] * 10 + [2] * 10, np.int32)
    X = np.abs(rng.standard_normal((21, 4))).astype(np.float32) + 0.5
    cols, rows = np.nonzero(X.T)  # column-major order = CSC order
    idp = np.searchsorted(cols, np.arange(5)).astype(np.int64)
    save("err_ref_small", X[rows, cols], rows.astype(np.int64), idp, gid_small_ref, 2, o_min)
    gid_small_tar = np.array([0] * 10 + [1] * 10 + [2], np.int32)
    save("err_target_small", X[rows, cols], rows.astype(np.int64), idp, gid_small_tar, 2, o_min)
    o_none = dict(o_min, zero_handling=0)
    Xn = X.copy()
    Xn[12:, 2] = 0.0   # column 2: target 1 keeps too few explicit values
    cols, rows = np.nonzero(Xn.T)
    idp = np.searchsorted(cols, np.arange(5)).astype(np.int64)
    gid3 = np.array([0] * 10 + [1] * 5 + [2] * 6, np.int32)
    save("err_none_column", Xn[rows, cols], rows.astype(np.int64), idp, gid3, 2, o_none)
    written += ["err_ref_small", "err_target_small", "err_none_column"]
    # 3d) heavy ties: integral counts with a handful of distinct values
    data, indices, indptr, gid = random_case(rng, 400, 8, 6, np.float32, 0.6, False, True, False)
    data = np.floor(np.abs(data) * 2.0).astype(np.float32) + 1.0
    save("edge_heavy_ties", data, indices, indptr, gid, 6, o_min)
    written.append("edge_heavy_ties")

    # 4) scaled-down copies of the large workloads
    w = synthetic.umi_counts(seed=5, n_rows=3000, n_cols=60, n_targets=12)
    save("umi_counts_small", w.data, w.indices, w.indptr, w.group_id, w.n_targets, o_min)
    w = synthetic.perturb_screen(seed=9, n_rows=6000, n_cols=120, n_targets=30, ref_size=600)
    save("perturb_screen_small", w.data, w.indices, w.indptr, w.group_id, w.n_targets, o_min)
    w = synthetic.exact_small(seed=3, n_rows=600, n_cols=12, n_targets=20, ref_size=12)
    o_exact = dict(tie_correction=True, use_continuity=False, zero_handling=0, alternative=2,
                   method=1)
    save("exact_small_small", w.data, w.indices, w.indptr, w.group_id, w.n_targets, o_exact)
    written += ["umi_counts_small", "perturb_screen_small", "exact_small_small"]

    extreme_shift()  # outputs only; not in the manifest of input+output fixtures

    with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
        json.dump(sorted(written), f, indent=0)
    print(f"wrote {len(written)} fixtures")


if __name__ == "__main__":
    main()
