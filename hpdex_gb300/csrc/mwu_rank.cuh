// mwu_rank.cuh -- per-gene rank-sum kernel of the Mann-Whitney U backend (sm_103a).
//
// One CTA owns one gene (CSC column) at a time; persistent CTAs pull genes from a device
// work queue in descending-nnz order (or take one fixed gene in the plain form). For the
// gene it computes, for every target g, the exact integers
//     2*U2[g] = sum over target elements x of (2 * #ref{< x} + #ref{== x})  (+ zero block)
//     tie[g]  = sum over distinct values of (t^3 - t) in ref u target g
// and writes U1 = n1*n2 - U2 and the (masked) tie sum; the p-value kernel finishes.
// This reproduces the reference's per-(gene, target) merge (AI4Cell/hpdex
// src/cpp/mannwhitneyu.cpp:618-840, driver :843-1065) without re-walking the reference
// slice for every target: the reference slice is ranked once per gene through a bucket
// index and every target element looks its rank up.
//
// Per gene:
//   pass 0  min/max of the order-preserving keys of stored values (value test only)
//   pass 1  value-bucket histograms: all stored elements and reference elements; per-group
//           stored counts (and negatives for zero_handling=mix)
//   scan    exclusive prefix sums -> bucket start, reference count below each bucket
//   pass 2  scatter (key, group) into bucket order (shared memory when it fits, else the
//           CTA's slice of a global scratch buffer that stays in L2)
//   rank    singleton buckets: one atomic; buckets <= SMALL: each element scans its bucket;
//           larger buckets: a warp checks purity (all keys equal), sorts impure ones, and
//           resolves each run of equal keys with per-warp group counters
//   final   zero block, U1, tie sum per target
//
// "Stored" elements are what the reference gathers into its slices (mannwhitneyu.cpp:
// 914-926): row id in [0, n_rows), group in [0, G), finite value; for zero_handling
// min/max/mix explicit zeros are left out too and join the implicit-zero block, whose size
// per group is group_rows[g] - stored[g] (:967-1003).
#pragma once
#include <climits>
#include <cstdint>

#include "common.cuh"

namespace hpdex {

struct RankArgs {
    const void* data;          // values of the CSC matrix (dtype V)
    const int32_t* rows;       // row ids (int32)
    const int64_t* indptr;     // [n_cols + 1]
    int64_t n_rows;
    int32_t n_cols;
    int32_t G;                 // n_targets + 1
    const int32_t* gid;        // [n_rows]
    const int32_t* order;      // genes in processing order [n_cols]
    int32_t* queue;            // work counter (batched form)
    int32_t single_gene;       // >= 0: plain form, this gene only
    int32_t zero_handling;
    int32_t tie_correction;
    const long long* group_rows;  // [G]
    double* U1;                // [T * n_cols] target-major
    double* tie;               // [T * n_cols] (the P buffer, overwritten later)
    uint32_t* n1;              // [n_cols]      zero_handling = none only
    uint32_t* n2;              // [T * n_cols]  zero_handling = none only
    unsigned long long* err;   // [0]: min(gene*G + group) of a too-small sample (none)
                               // [1]: min(gene*G + group) of a group with more stored
                               //      entries than rows (duplicate row ids)
    // global scratch, one slice of `slice` elements per CTA
    void* ek_global;
    uint32_t* eg_global;
    void* tk_global;
    uint32_t* tg_global;
    long long slice;
    unsigned char* acc_global; // per CTA 24*G bytes when the accumulators are not in SMEM
    uint32_t* tiecnt_global;   // per CTA tie_warps*G when the counters are not in SMEM
    int32_t nb_max_log2;       // bucket table capacity (power of two)
    int32_t elem_smem_cap;     // elements that fit in shared memory
    int32_t acc_in_smem;
    int32_t tiecnt_in_smem;
    int32_t tie_warps;
};

constexpr int kSmallBucket = 16;

// Shared-memory layout shared by host (sizing) and device (carving).
struct RankSmem {
    size_t hist_bytes, acc_bytes, tiecnt_bytes, elem_bytes, total;
    __host__ __device__ static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
    __host__ __device__ RankSmem(int nb_max_log2, int G, int tie_warps, int acc_in_smem,
                                 int tiecnt_in_smem, int elem_cap, int key_bytes) {
        const size_t NB = size_t(1) << nb_max_log2;
        hist_bytes = align16((3 * NB + 2) * 4);
        acc_bytes = acc_in_smem ? align16(size_t(G) * 24) : 0;
        tiecnt_bytes = tiecnt_in_smem ? align16(size_t(tie_warps) * G * 4) : 0;
        elem_bytes = align16(size_t(elem_cap) * (key_bytes + 4));
        total = hist_bytes + acc_bytes + tiecnt_bytes + elem_bytes;
    }
};

template <int NT>
__device__ void block_scan2(uint32_t* x, uint32_t* y, int L, uint32_t* wsx, uint32_t* wsy) {
    // exclusive prefix sums of x[0..L) and y[0..L) in place; x[L], y[L] = totals
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (L + NT - 1) / NT;
    const int beg = min(L, tid * per), end = min(L, beg + per);
    uint32_t sx = 0, sy = 0;
    for (int i = beg; i < end; ++i) { sx += x[i]; sy += y[i]; }
    const uint32_t ix = warp_incl_scan(sx), iy = warp_incl_scan(sy);
    if (lane == 31) { wsx[warp] = ix; wsy[warp] = iy; }
    __syncthreads();
    if (warp == 0) {
        const uint32_t vx = lane < NT / 32 ? wsx[lane] : 0u;
        const uint32_t vy = lane < NT / 32 ? wsy[lane] : 0u;
        const uint32_t px = warp_incl_scan(vx), py = warp_incl_scan(vy);
        if (lane < NT / 32) { wsx[lane] = px - vx; wsy[lane] = py - vy; }
        if (lane == 31) { x[L] = px; y[L] = py; }
    }
    __syncthreads();
    uint32_t ox = wsx[warp] + ix - sx, oy = wsy[warp] + iy - sy;
    for (int i = beg; i < end; ++i) {
        const uint32_t tx = x[i], ty = y[i];
        x[i] = ox; ox += tx;
        y[i] = oy; oy += ty;
    }
    __syncthreads();
}

// A run of equal keys [start, start+len) inside a bucket: every element shares the value.
// lref = reference elements below the run, c0 = reference elements in the run.
template <class K>
__device__ __forceinline__ void resolve_run(const uint32_t* gptr, uint32_t start, uint32_t len,
                                            unsigned long long lref, unsigned long long c0,
                                            unsigned long long* A, unsigned long long* B,
                                            uint32_t* cnt, unsigned long long& tref) {
    const int lane = threadIdx.x & 31;
    if (len == 1) {
        if (lane == 0) {
            const uint32_t g = gptr[start];
            if (g) atomicAdd(&A[g], 2ull * lref);  // a lone target value: c0 = 0
        }
        return;
    }
    for (uint32_t j = lane; j < len; j += 32) {
        const uint32_t g = gptr[start + j];
        if (g) atomicAdd(&cnt[g], 1u);
    }
    __syncwarp();
    const unsigned long long a = 2ull * lref + c0;
    for (uint32_t j = lane; j < len; j += 32) {
        const uint32_t g = gptr[start + j];
        if (g) {
            const unsigned long long s = cnt[g];
            atomicAdd(&A[g], a);
            // per-element share of (c0+s)^3-(c0+s) - (c0^3-c0) over the s equal values
            const unsigned long long tb = 3ull * c0 * c0 + 3ull * c0 * s + s * s - 1ull;
            if (tb) atomicAdd(&B[g], tb);
        }
    }
    __syncwarp();
    for (uint32_t j = lane; j < len; j += 32) {
        const uint32_t g = gptr[start + j];
        if (g) cnt[g] = 0u;
    }
    __syncwarp();
    if (lane == 0) tref += c0 * c0 * c0 - c0;
}

// Warp-level handling of a bucket with more than kSmallBucket elements.
template <class K>
__device__ void resolve_big_bucket(uint32_t b, const uint32_t* hall, const uint32_t* href,
                                   const K* ek, const uint32_t* eg, K* tk, uint32_t* tg,
                                   unsigned long long* A, unsigned long long* B, uint32_t* cnt,
                                   unsigned long long& tref) {
    const int lane = threadIdx.x & 31;
    const uint32_t s0 = hall[b], m = hall[b + 1] - s0;
    const uint32_t rb = href[b], c0b = href[b + 1] - rb;
    K lo = ~K(0), hi = K(0);
    for (uint32_t j = lane; j < m; j += 32) {
        const K k = ek[s0 + j];
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
    }
    lo = warp_min(lo);
    hi = warp_max(hi);
    if (lo == hi) {  // pure bucket: one run holding every element
        resolve_run<K>(eg, s0, m, rb, c0b, A, B, cnt, tref);
        return;
    }
    // impure: order the bucket by key (rank placement into the temp slice), then walk runs
    for (uint32_t i = lane; i < m; i += 32) {
        const K k = ek[s0 + i];
        uint32_t r = 0;
        for (uint32_t j = 0; j < m; ++j) {
            const K kj = ek[s0 + j];
            r += (kj < k) || (kj == k && j < i);
        }
        tk[s0 + r] = k;
        tg[s0 + r] = eg[s0 + i];
    }
    __syncwarp();
    uint32_t pos = 0;
    unsigned long long lref = rb;
    while (pos < m) {
        const K key = tk[s0 + pos];
        uint32_t end = m;
        for (uint32_t base = pos; base < m; base += 32) {
            const uint32_t j = base + lane;
            const bool diff = (j < m) && (tk[s0 + j] != key);
            const unsigned msk = __ballot_sync(0xffffffffu, diff);
            if (msk) { end = base + (uint32_t)(__ffs((int)msk) - 1); break; }
        }
        uint32_t c0 = 0;
        for (uint32_t j = pos + lane; j < end; j += 32) c0 += (tg[s0 + j] == 0u);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) c0 += __shfl_xor_sync(0xffffffffu, c0, d);
        resolve_run<K>(tg, s0 + pos, end - pos, lref, c0, A, B, cnt, tref);
        lref += c0;
        pos = end;
    }
    __syncwarp();
}

template <class V, int NT>
__global__ void __launch_bounds__(NT) mwu_rank_kernel(const RankArgs a) {
    using K = typename Val<V>::Key;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_gene;
    __shared__ K s_kmin, s_kmax;
    __shared__ unsigned long long s_tref;
    __shared__ uint32_t s_nbig;
    __shared__ uint32_t s_wsx[32], s_wsy[32];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int G = a.G, zh = a.zero_handling;
    const int NBMAX = 1 << a.nb_max_log2;
    const RankSmem L(a.nb_max_log2, G, a.tie_warps, a.acc_in_smem, a.tiecnt_in_smem,
                     a.elem_smem_cap, (int)sizeof(K));

    uint32_t* hall = reinterpret_cast<uint32_t*>(smem);
    uint32_t* href = hall + NBMAX + 1;
    uint32_t* cursor = href + NBMAX + 1;
    unsigned char* accb = a.acc_in_smem ? smem + L.hist_bytes
                                        : a.acc_global + (size_t)blockIdx.x * 24 * G;
    unsigned long long* A = reinterpret_cast<unsigned long long*>(accb);
    unsigned long long* B = A + G;
    uint32_t* nz = reinterpret_cast<uint32_t*>(B + G);
    uint32_t* ng = nz + G;
    uint32_t* tiecnt = a.tiecnt_in_smem
                           ? reinterpret_cast<uint32_t*>(smem + L.hist_bytes + L.acc_bytes)
                           : a.tiecnt_global + (size_t)blockIdx.x * a.tie_warps * G;
    K* ek_s = reinterpret_cast<K*>(smem + L.hist_bytes + L.acc_bytes + L.tiecnt_bytes);
    uint32_t* eg_s = reinterpret_cast<uint32_t*>(ek_s + a.elem_smem_cap);
    K* ek_g = reinterpret_cast<K*>(a.ek_global) + (size_t)blockIdx.x * a.slice;
    uint32_t* eg_g = a.eg_global + (size_t)blockIdx.x * a.slice;
    K* tk = reinterpret_cast<K*>(a.tk_global) + (size_t)blockIdx.x * a.slice;
    uint32_t* tg = a.tg_global + (size_t)blockIdx.x * a.slice;

    const V* data = reinterpret_cast<const V*>(a.data);
    const int32_t* rows = a.rows;

    for (int i = tid; i < a.tie_warps * G; i += NT) tiecnt[i] = 0u;

    bool first = true;
    for (;;) {
        if (tid == 0) {
            int c = -1;
            if (a.single_gene >= 0) {
                c = first ? a.single_gene : -1;
            } else {
                const int gi = atomicAdd(a.queue, 1);
                c = gi < a.n_cols ? a.order[gi] : -1;
            }
            s_gene = c;
            s_kmin = ~K(0);
            s_kmax = K(0);
            s_tref = 0ull;
            s_nbig = 0u;
        }
        first = false;
        for (int g = tid; g < G; g += NT) { A[g] = 0ull; B[g] = 0ull; nz[g] = 0u; ng[g] = 0u; }
        __syncthreads();
        const int c = s_gene;
        if (c < 0) break;
        const long long p0 = a.indptr[c], p1 = a.indptr[c + 1];

        // ---- pass 0: key range of candidate values ----
        {
            K lo = ~K(0), hi = K(0);
            for (long long p = p0 + tid; p < p1; p += NT) {
                const V v = data[p];
                if (Val<V>::finite(v) && (zh == ZH_NONE || !Val<V>::zero(v))) {
                    const K k = Val<V>::key(v);
                    lo = k < lo ? k : lo;
                    hi = k > hi ? k : hi;
                }
            }
            lo = warp_min(lo);
            hi = warp_max(hi);
            if (lane == 0 && lo <= hi) {
                atomicMin(&s_kmin, lo);
                atomicMax(&s_kmax, hi);
            }
        }
        __syncthreads();
        const K kmin = s_kmin, kmax = s_kmax;
        const long long nraw = p1 - p0;
        int nbl = 1;
        while (nbl < a.nb_max_log2 && (1ll << nbl) < nraw) ++nbl;
        const int NB = 1 << nbl;
        int shift = 0;
        if (kmin <= kmax) {
            const int bl = bit_length(K(kmax - kmin));
            shift = bl > nbl ? bl - nbl : 0;
        }
        for (int b = tid; b <= NB; b += NT) { hall[b] = 0u; href[b] = 0u; }
        __syncthreads();

        // ---- pass 1: histograms and per-group stored counts ----
        for (long long p = p0 + tid; p < p1; p += NT) {
            const long long r = rows[p];
            if (r < 0 || r >= a.n_rows) continue;
            const int g = a.gid[r];
            if (g < 0 || g >= G) continue;
            const V v = data[p];
            if (!Val<V>::finite(v)) continue;
            if (zh != ZH_NONE && Val<V>::zero(v)) continue;
            atomicAdd(&nz[g], 1u);
            if (zh == ZH_MIX && Val<V>::neg(v)) atomicAdd(&ng[g], 1u);
            const uint32_t b = (uint32_t)((Val<V>::key(v) - kmin) >> shift);
            atomicAdd(&hall[b], 1u);
            if (g == 0) atomicAdd(&href[b], 1u);
        }
        __syncthreads();
        block_scan2<NT>(hall, href, NB, s_wsx, s_wsy);
        const uint32_t n = hall[NB];
        for (int b = tid; b < NB; b += NT) cursor[b] = hall[b];
        K* ek = (n <= (uint32_t)a.elem_smem_cap) ? ek_s : ek_g;
        uint32_t* eg = (n <= (uint32_t)a.elem_smem_cap) ? eg_s : eg_g;
        __syncthreads();

        // ---- pass 2: scatter into bucket order ----
        for (long long p = p0 + tid; p < p1; p += NT) {
            const long long r = rows[p];
            if (r < 0 || r >= a.n_rows) continue;
            const int g = a.gid[r];
            if (g < 0 || g >= G) continue;
            const V v = data[p];
            if (!Val<V>::finite(v)) continue;
            if (zh != ZH_NONE && Val<V>::zero(v)) continue;
            const K k = Val<V>::key(v);
            const uint32_t b = (uint32_t)((k - kmin) >> shift);
            const uint32_t pos = atomicAdd(&cursor[b], 1u);
            ek[pos] = k;
            eg[pos] = (uint32_t)g;
        }
        __syncthreads();

        // ---- rank: singletons and small buckets per element ----
        unsigned long long tref = 0ull;
        for (uint32_t i = tid; i < n; i += NT) {
            const K k = ek[i];
            const uint32_t g = eg[i];
            const uint32_t b = (uint32_t)((k - kmin) >> shift);
            const uint32_t s0 = hall[b], m = hall[b + 1] - s0, rb = href[b];
            if (m == 1) {
                if (g) atomicAdd(&A[g], 2ull * rb);
            } else if (m <= (uint32_t)kSmallBucket) {
                uint32_t lt = 0, c0 = 0, s = 0;
                for (uint32_t j = s0; j < s0 + m; ++j) {
                    const K kj = ek[j];
                    const uint32_t gj = eg[j];
                    if (gj == 0u) { lt += (kj < k); c0 += (kj == k); }
                    s += (gj == g && kj == k);
                }
                if (g) {
                    atomicAdd(&A[g], 2ull * (rb + lt) + c0);
                    const unsigned long long c = c0, ss = s;
                    const unsigned long long tb = 3ull * c * c + 3ull * c * ss + ss * ss - 1ull;
                    if (tb) atomicAdd(&B[g], tb);
                } else {
                    tref += (unsigned long long)c0 * c0 - 1ull;
                }
            } else if (i == s0) {
                cursor[atomicAdd(&s_nbig, 1u)] = b;
            }
        }
        __syncthreads();  // the big-bucket list in `cursor` is complete

        // ---- rank: big buckets, one warp each ----
        if (warp < a.tie_warps) {
            uint32_t* cnt = tiecnt + (size_t)warp * G;
            const uint32_t nbig = s_nbig;
            for (uint32_t q = warp; q < nbig; q += a.tie_warps)
                resolve_big_bucket<K>(cursor[q], hall, href, ek, eg, tk, tg, A, B, cnt, tref);
        }
        tref = warp_sum_u64(tref);
        if (lane == 0 && tref) atomicAdd(&s_tref, tref);
        __syncthreads();

        // ---- finalize per target ----
        const unsigned long long T_ref = s_tref;
        const unsigned long long nz1 = nz[0];
        const int T = G - 1;
        for (int g = 1 + tid; g < G; g += NT) {
            const size_t idx = (size_t)(g - 1) * a.n_cols + c;
            const unsigned long long nz2 = nz[g];
            unsigned long long n1, n2, u2x2, ties;
            if (zh == ZH_NONE) {
                n1 = nz1;
                n2 = nz2;
                if (n1 < 2) atomicMin(&a.err[0], (unsigned long long)c * G);
                else if (n2 < 2) atomicMin(&a.err[0], (unsigned long long)c * G + g);
                u2x2 = A[g];
                ties = T_ref + B[g];
                a.n2[idx] = (uint32_t)nz2;
                if (g == 1) a.n1[c] = (uint32_t)nz1;
            } else {
                n1 = (unsigned long long)a.group_rows[0];
                n2 = (unsigned long long)a.group_rows[g];
                if (nz1 > n1) atomicMin(&a.err[1], (unsigned long long)c * G);
                if (nz2 > n2) atomicMin(&a.err[1], (unsigned long long)c * G + g);
                const unsigned long long z1 = n1 - nz1, z2 = n2 - nz2;
                if (zh == ZH_MIN) u2x2 = A[g] + 2ull * z1 * nz2 + z1 * z2;
                else if (zh == ZH_MAX) u2x2 = A[g] + z2 * (2ull * nz1 + z1);
                else u2x2 = A[g] + 2ull * z1 * (nz2 - ng[g]) + z2 * (2ull * ng[0] + z1);
                const unsigned long long zz = z1 + z2;
                ties = T_ref + B[g] + zz * zz * zz - zz;
            }
            const long long u1x2 = (long long)(2ull * n1 * n2) - (long long)u2x2;
            a.U1[idx] = (double)u1x2 * 0.5;
            a.tie[idx] = a.tie_correction ? (double)ties : 0.0;
        }
        (void)T;
        __syncthreads();
    }
}

}  // namespace hpdex
