"""CPU restatement of the rank kernel's warp rounds (resolve_round in mwu_rank.cuh): up to 32
lanes hold whole buckets of 2..32 elements; each target lane adds 2*(rb + lt) + c0 to A[g] and
3*c0^2 + 3*c0*s + s^2 - 1 to B[g], each reference lane c0^2 - 1 to the reference tie sum, where
lt / c0 count the reference elements of its bucket with a smaller / equal key and s the target
elements with its bucket, key and group.

The kernel finds lt, c0 and s in two ways, both restated here lane by lane, with inactive lanes
holding garbage as in the kernel:
- counters (run counters in shared memory): one-key buckets take c0 = their reference lanes and
  lt = 0; the warp's group counters give ng, the lanes of the round with the same group; lanes
  of one-key buckets whose group repeats match their group among themselves, lanes of buckets
  with several keys compare pairwise among themselves;
- warp match (run counters in global memory): one match over the target lanes' groups gives ng
  and, in one-key buckets, s.
Both must equal the pairwise definition, and the per-lane shares summed over a (key, group) run
must equal the run-level terms s * (2 * lref + c0) and (c0 + s)^3 - (c0 + s) - (c0^3 - c0)."""
import numpy as np


def _round(rng):
    """A packed round: whole buckets of 2..11 elements with 1-3 keys and groups 0..4 (0 is the
    reference), the rest of the 32 lanes inactive with garbage."""
    sizes, tot = [], 0
    while True:
        m = int(rng.integers(2, 12))
        if tot + m > 32:
            break
        sizes.append(m)
        tot += m
        if rng.random() < 0.2:
            break
    key = np.zeros(32, np.int64)
    g = np.zeros(32, np.int64)
    sub = np.zeros(32, np.int64)
    active = np.zeros(32, bool)
    p = 0
    for m in sizes:
        nk = int(rng.integers(1, 4))
        key[p:p + m] = rng.integers(0, nk, size=m) + 100
        g[p:p + m] = rng.integers(0, 5, size=m)
        sub[p:p + m] = ((1 << m) - 1) << p
        active[p:p + m] = True
        p += m
    key[p:] = rng.integers(0, 5, size=32 - p)
    g[p:] = rng.integers(0, 4, size=32 - p)
    sub[p:] = rng.integers(0, 2 ** 32, size=32 - p)
    return key, g, sub, active


def _bits(mask):
    return [j for j in range(32) if (mask >> j) & 1]


def _popc(x):
    return bin(int(x)).count("1")


def _definition(key, g, sub, active):
    lt = np.zeros(32, int)
    c0 = np.zeros(32, int)
    s = np.ones(32, int)
    for L in range(32):
        if not active[L]:
            continue
        same_bucket = [j for j in range(32) if (int(sub[L]) >> j) & 1]
        lt[L] = sum(1 for j in same_bucket if g[j] == 0 and key[j] < key[L])
        c0[L] = sum(1 for j in same_bucket if g[j] == 0 and key[j] == key[L])
        if g[L] != 0:
            s[L] = sum(1 for j in same_bucket if g[j] == g[L] and key[j] == key[L])
    return lt, c0, s


def _kernel(key, g, sub, active, match):
    is_ref = active & (g == 0)
    is_tar = active & (g != 0)
    refm = sum(1 << L for L in range(32) if is_ref[L])
    first = [(int(sub[L]) & -int(sub[L])).bit_length() - 1 if active[L] else L for L in range(32)]
    diff = sum(1 << L for L in range(32) if active[L] and key[L] != key[first[L]])
    mixed = [(int(sub[L]) & diff) != 0 for L in range(32)]
    mixm = sum(1 << L for L in range(32) if active[L] and mixed[L])
    lt = np.zeros(32, int)
    c0 = np.array([0 if mixed[L] else _popc(refm & int(sub[L])) for L in range(32)])
    for j in _bits(refm & mixm):  # reference lanes of buckets with several keys, broadcast
        for L in range(32):
            if (int(sub[L]) >> j) & 1:
                lt[L] += key[j] < key[L]
                c0[L] += key[j] == key[L]
    s = np.ones(32, int)
    if match:
        val = [int(g[L]) if is_tar[L] else (0x80000000 | L) for L in range(32)]
        same = [sum(1 << j for j in range(32) if val[j] == val[L]) for L in range(32)]
        ng = [_popc(same[L]) if is_tar[L] else 0 for L in range(32)]
        for L in range(32):
            if ng[L] > 1 and not mixed[L]:
                s[L] = _popc(same[L] & int(sub[L]))
        repeats = True
    else:
        ng = [int((is_tar & (g == g[L])).sum()) if is_tar[L] else 0 for L in range(32)]
        repeats = any(n > 1 for n in ng)
        if repeats:
            one = sum(1 << L for L in range(32) if ng[L] > 1 and not mixed[L])
            for L in range(32):
                if (one >> L) & 1:
                    m = sum(1 << j for j in _bits(one) if g[j] == g[L])
                    s[L] = _popc(m & int(sub[L]))
    if repeats:
        many = sum(1 << L for L in range(32) if ng[L] > 1 and mixed[L])
        for L in range(32):
            if ng[L] > 1 and mixed[L]:
                s[L] = sum(1 for j in _bits(many)
                           if (int(sub[L]) >> j) & 1 and g[j] == g[L] and key[j] == key[L])
    return lt, c0, s


def test_round_resolution_equals_the_definition():
    rng = np.random.default_rng(3)
    for _ in range(3000):
        key, g, sub, active = _round(rng)
        lt_d, c0_d, s_d = _definition(key, g, sub, active)
        for match in (False, True):
            lt, c0, s = _kernel(key, g, sub, active, match)
            for L in range(32):
                if active[L]:
                    assert (lt[L], c0[L]) == (lt_d[L], c0_d[L])
                if active[L] and g[L] != 0:
                    assert s[L] == s_d[L]


def test_lane_shares_sum_to_the_run_terms():
    """Over a run of s target elements of one group with c0 reference elements of equal key and
    lref below, the lanes' shares add up to the merge's terms (reference mannwhitneyu.cpp:618-659)."""
    for c0 in range(0, 12):
        for s in range(1, 12):
            for lref in (0, 7, 1000):
                a = sum(2 * (lref) + c0 for _ in range(s))
                b = sum(3 * c0 * c0 + 3 * c0 * s + s * s - 1 for _ in range(s))
                assert a == s * (2 * lref + c0)
                assert b == (c0 + s) ** 3 - (c0 + s) - (c0 ** 3 - c0)
            # reference lanes: c0 of them, each adding c0^2 - 1
            assert sum(c0 * c0 - 1 for _ in range(c0)) == c0 ** 3 - c0
