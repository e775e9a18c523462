"""The rank kernel's integer formulation, restated in numpy and checked against the oracle.

The reference ranks by sorting each group's values as doubles and merging (mannwhitneyu.cpp
:618-840), with the zero block placed by zero_handling (:662-788). The CUDA rank kernel
(hpdex_gb300/csrc/mwu_rank.cuh) never sorts or merges: per gene and target it counts, for
every stored nonzero target value x, the reference values below and equal to x, and adds
closed-form terms for the zero block (implicit zeros, explicit zeros and non-finite values,
z_g = group_rows[g] - stored nonzero of g):

    2 U2 = sum_x (2 #ref{< x} + #ref{== x}) + Z
    Z    = 2 z1 nz2 + z1 z2                      (min: zeros below everything)
         = z2 (2 nz1 + z1)                       (max: zeros above everything)
         = 2 z1 (nz2 - neg2) + z2 (2 neg1 + z1)  (mix: zeros between negatives and positives)
    U1   = n1 n2 - U2
    tie  = T_ref + sum_{distinct target v} [(r_v + s_v)^3 - (r_v + s_v) - (r_v^3 - r_v)]
           + (z1 + z2)^3 - (z1 + z2)

with T_ref = sum over distinct reference values of r^3 - r, once per gene. In mode none only
finite stored values take part (explicit zeros included) and there is no zero block. All of it
is integer arithmetic, hence U1 and the tie sum bit-exact against the reference's double
sums (exact below 2^53).

The second restatement is the per-element form (a candidate for a later rank kernel): each
stored target element of value v, arriving as the i-th (0-based) of its (v, group) run, adds
2 R_<v + r_v to 2 U2 and 3 r_v^2 + 3 r_v (2 i + 1) + 3 i (i + 1) to the tie sum, in any
arrival order; summed over a run of s elements that is the bracket above.

Both are compared with the oracle's (U1, n1, n2, tie) on seeded data with heavy ties, explicit
zeros, negatives, NaN and infinities, rows in no group and out-of-range row ids, in all four
zero modes. Bar: exact equality.
"""
import numpy as np
import pytest

ZH = {"none": 0, "min": 1, "max": 2, "mix": 3}


def _data(seed, n_rows=400, n_cols=30, n_targets=6):
    rng = np.random.default_rng(seed)
    gid = rng.integers(-1, n_targets + 2, size=n_rows).astype(np.int32)  # -1 and > T: no group
    gid[: 2 * (n_targets + 1)] = np.repeat(np.arange(n_targets + 1), 2)  # every group >= 2 rows
    cols_d, cols_i, ptr = [], [], [0]
    for c in range(n_cols):
        k = int(rng.integers(0, n_rows))
        rows = np.sort(rng.choice(n_rows, size=k, replace=False)).astype(np.int64)
        vals = rng.integers(-4, 9, size=k).astype(np.float64)  # heavy ties, negatives, zeros
        if c % 3 == 0:
            vals = vals + rng.integers(0, 3, size=k) * 0.25
        bad = rng.random(k)
        vals[bad < 0.02] = np.nan
        vals[(bad >= 0.02) & (bad < 0.03)] = np.inf
        vals[(bad >= 0.03) & (bad < 0.04)] = -np.inf
        rows[rng.random(k) < 0.02] = n_rows + 5  # out of range: skipped
        cols_d.append(vals)
        cols_i.append(rows)
        ptr.append(ptr[-1] + k)
    return (np.concatenate(cols_d), np.concatenate(cols_i), np.asarray(ptr, np.int64), gid,
            n_rows, n_targets)


def _gather(data, indices, indptr, gid, n_rows, c):
    v = data[indptr[c]:indptr[c + 1]]
    r = indices[indptr[c]:indptr[c + 1]]
    ok = (r >= 0) & (r < n_rows)
    v, r = v[ok], r[ok]
    return v, gid[r]


def _kernel_form(data, indices, indptr, gid, n_rows, T, zh):
    C = indptr.size - 1
    group_rows = np.bincount(gid[(gid >= 0) & (gid <= T)], minlength=T + 1).astype(np.int64)
    U1 = np.zeros((T, C))
    tie = np.zeros((T, C))
    for c in range(C):
        v, g = _gather(data, indices, indptr, gid, n_rows, c)
        keep = np.isfinite(v) & (g >= 0) & (g <= T)
        if zh != "none":
            keep &= v != 0.0
        v, g = v[keep], g[keep]
        a = np.sort(v[g == 0])
        ua, ra = np.unique(a, return_counts=True)
        t_ref = int(np.sum(ra.astype(np.int64) ** 3 - ra))
        ref_count = dict(zip(ua.tolist(), ra.tolist()))
        for t in range(1, T + 1):
            b = v[g == t]
            lt = np.searchsorted(a, b, side="left").astype(np.int64)
            eq = np.searchsorted(a, b, side="right").astype(np.int64) - lt
            two_u2 = int(np.sum(2 * lt + eq))
            if zh == "none":
                n1, n2, z1, z2 = a.size, b.size, 0, 0
            else:
                n1, n2 = int(group_rows[0]), int(group_rows[t])
                z1, z2 = n1 - a.size, n2 - b.size
                nz1, nz2 = a.size, b.size
                if zh == "min":
                    two_u2 += 2 * z1 * nz2 + z1 * z2
                elif zh == "max":
                    two_u2 += z2 * (2 * nz1 + z1)
                else:
                    neg1, neg2 = int(np.sum(a < 0)), int(np.sum(b < 0))
                    two_u2 += 2 * z1 * (nz2 - neg2) + z2 * (2 * neg1 + z1)
            ub, sb = np.unique(b, return_counts=True)
            r = np.array([ref_count.get(x, 0) for x in ub.tolist()], np.int64)
            s = sb.astype(np.int64)
            ts = t_ref + int(np.sum((r + s) ** 3 - (r + s) - (r ** 3 - r)))
            z = z1 + z2
            ts += z ** 3 - z
            U1[t - 1, c] = (2 * n1 * n2 - two_u2) / 2
            tie[t - 1, c] = ts
    return U1, tie


def _per_element_form(data, indices, indptr, gid, n_rows, T, zh, seed):
    """Zero-block terms as in the kernel form; stored target elements one at a time, in a
    random arrival order, with a per-(value, group) arrival counter."""
    rng = np.random.default_rng(seed)
    C = indptr.size - 1
    group_rows = np.bincount(gid[(gid >= 0) & (gid <= T)], minlength=T + 1).astype(np.int64)
    U1 = np.zeros((T, C))
    tie = np.zeros((T, C))
    for c in range(C):
        v, g = _gather(data, indices, indptr, gid, n_rows, c)
        keep = np.isfinite(v) & (g >= 0) & (g <= T)
        if zh != "none":
            keep &= v != 0.0
        v, g = v[keep], g[keep]
        a = np.sort(v[g == 0])
        ua, ra = np.unique(a, return_counts=True)
        t_ref = int(np.sum(ra.astype(np.int64) ** 3 - ra))
        ref_count = dict(zip(ua.tolist(), ra.tolist()))
        two_u2 = np.zeros(T + 1, np.int64)
        ts = np.full(T + 1, t_ref, np.int64)
        seen = {}
        for k in rng.permutation(np.nonzero(g > 0)[0]):
            x, t = float(v[k]), int(g[k])
            r = ref_count.get(x, 0)
            below = int(np.searchsorted(a, x, side="left"))
            two_u2[t] += 2 * below + r
            i = seen.get((x, t), 0)
            seen[(x, t)] = i + 1
            ts[t] += 3 * r * r + 3 * r * (2 * i + 1) + 3 * i * (i + 1)
        for t in range(1, T + 1):
            nb = int(np.sum(g == t))
            if zh == "none":
                n1, n2, z1, z2 = a.size, nb, 0, 0
                zt = 0
            else:
                n1, n2 = int(group_rows[0]), int(group_rows[t])
                z1, z2 = n1 - a.size, n2 - nb
                nz1, nz2 = a.size, nb
                if zh == "min":
                    zt = 2 * z1 * nz2 + z1 * z2
                elif zh == "max":
                    zt = z2 * (2 * nz1 + z1)
                else:
                    neg1, neg2 = int(np.sum(a < 0)), int(np.sum(v[g == t] < 0))
                    zt = 2 * z1 * (nz2 - neg2) + z2 * (2 * neg1 + z1)
            z = z1 + z2
            U1[t - 1, c] = (2 * n1 * n2 - (two_u2[t] + zt)) / 2
            tie[t - 1, c] = ts[t] + z ** 3 - z
    return U1, tie


def _oracle(data, indices, indptr, gid, T, zh):
    from oracle import oracle
    U1, n1, n2, tie = oracle.mwu_stats(data, indices, indptr, gid, T, ZH[zh])
    C = indptr.size - 1
    return U1.reshape(C, T).T, tie.reshape(C, T).T


@pytest.mark.parametrize("zh", ["none", "min", "max", "mix"])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_kernel_formulation_equals_oracle(zh, seed):
    data, indices, indptr, gid, n_rows, T = _data(seed)
    U1o, tieo = _oracle(data, indices, indptr, gid, T, zh)
    U1, tie = _kernel_form(data, indices, indptr, gid, n_rows, T, zh)
    np.testing.assert_array_equal(U1, U1o)
    np.testing.assert_array_equal(tie, tieo)


@pytest.mark.parametrize("zh", ["none", "min", "mix"])
def test_per_element_formulation_equals_oracle(zh):
    data, indices, indptr, gid, n_rows, T = _data(11, n_rows=300, n_cols=12, n_targets=4)
    U1o, tieo = _oracle(data, indices, indptr, gid, T, zh)
    U1, tie = _per_element_form(data, indices, indptr, gid, n_rows, T, zh, seed=5)
    np.testing.assert_array_equal(U1, U1o)
    np.testing.assert_array_equal(tie, tieo)


def test_formulation_notices_a_planted_error():
    """The comparison is not vacuous: a zero block moved from below to above (min read as
    max) changes U1."""
    data, indices, indptr, gid, n_rows, T = _data(1)
    U1o, _ = _oracle(data, indices, indptr, gid, T, "min")
    U1, _ = _kernel_form(data, indices, indptr, gid, n_rows, T, "max")
    assert not np.array_equal(U1, U1o)
