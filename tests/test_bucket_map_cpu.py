"""CPU check of the rank kernel's signed bucket map (BucketMap in hpdex_gb300/csrc/mwu_rank.cuh),
restated in numpy for float32: for genes whose values take both signs the bucket of a value is
(m(x) - m(xmin)) >> shift with m linear in |x| below 2^E0 and following the float's bits above.
The kernel only needs the map to be non-decreasing in the value and to stay inside the bucket
table; a value outside it would index shared memory out of range. Checked on random genes over
80 decades, with subnormals, signed zeros and the values next to the linear/log junction, and
the bucket sizes it gives an N(0,1) gene against the plain key map."""
import numpy as np

NBL = 13


def key32(v):
    u = v.view(np.uint32).astype(np.uint64)
    u = np.where(((u << 1) & 0xFFFFFFFF) == 0, 0, u)  # -0.0 ties with +0.0
    return np.where(u & 0x80000000, (~u) & 0xFFFFFFFF, u | 0x80000000).astype(np.uint64)


def f32_of_key(k):
    k = k.astype(np.uint64)
    u = np.where(k & 0x80000000, k & 0x7FFFFFFF, (~k) & 0xFFFFFFFF).astype(np.uint32)
    return u.view(np.float32)


def e0_of(kmin, kmax):
    amag = min(abs(float(f32_of_key(np.array([kmin]))[0])), abs(float(f32_of_key(np.array([kmax]))[0])))
    ea = int(np.frexp(amag)[1])  # amag = f * 2^ea, f in [0.5, 1)
    return max(ea - 12, -100)


def m_of(k, e0):
    x = f32_of_key(k)
    t = np.abs(x)
    bits = t.view(np.uint32).astype(np.int64)
    b0 = (e0 + 127) << 23
    lin = np.float32(2.0) ** np.float32(23 - e0)
    with np.errstate(invalid="ignore", over="ignore"):
        lin_part = np.where(bits < b0, t * lin, 0).astype(np.uint32).astype(np.int64)
    u = np.where(bits >= b0, bits - b0 + (1 << 23), lin_part)
    return np.where(x < 0, 0x80000000 - u, 0x80000000 + u)


def buckets(v):
    k = key32(v)
    kmin, kmax = int(k.min()), int(k.max())
    e0 = e0_of(kmin, kmax)
    base, hi = int(m_of(np.array([kmin], np.uint64), e0)[0]), int(m_of(np.array([kmax], np.uint64), e0)[0])
    shift = max(0, (hi - base).bit_length() - NBL)
    return (m_of(k, e0) - base) >> shift, e0


def test_signed_map_is_monotone_and_in_range():
    rng = np.random.default_rng(1)
    for trial in range(150):
        scale = 10.0 ** rng.uniform(-40, 38)
        with np.errstate(over="ignore"):
            v = (rng.standard_normal(20_000) * scale * 10.0 ** rng.uniform(-2, 2, 20_000)).astype(np.float32)
        v = np.concatenate([v, np.array([-0.0, 1e-45, -1e-45, 1.1754944e-38, -3.0, 3.0], np.float32)])
        v = v[np.isfinite(v) & (v != 0)]
        if not (v.min() < 0 < v.max()):
            continue
        b, e0 = buckets(np.sort(v))
        assert np.all(np.diff(b) >= 0), trial  # sorted values give non-decreasing buckets
        assert b.min() == 0 and b.max() < (1 << NBL), trial
        j = np.float32(2.0) ** np.float32(e0)  # the junction of the two parts
        jj = np.array([-j, -np.nextafter(j, np.float32(0)), np.nextafter(j, np.float32(0)), j,
                       np.nextafter(j, np.float32(np.inf))], np.float32)
        mj = m_of(key32(jj), e0)
        assert np.all(np.diff(mj) >= 0), trial


def test_signed_map_spreads_a_normal_gene():
    v = np.random.default_rng(0).standard_normal(32_600).astype(np.float32)
    b, _ = buckets(v)
    cnt = np.bincount(b)
    k = key32(v).astype(np.int64)
    plain = np.bincount((k - k.min()) >> max(0, int(k.max() - k.min()).bit_length() - NBL))
    assert cnt.max() <= 64 and plain.max() > 400
    assert cnt[cnt > 32].sum() < 0.1 * v.size < plain[plain > 32].sum()
