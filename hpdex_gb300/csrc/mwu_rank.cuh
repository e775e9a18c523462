// mwu_rank.cuh -- per-gene rank-sum kernel of the Mann-Whitney U backend (sm_103a).
//
// One CTA owns one gene (CSC column) at a time; persistent CTAs (one per SM) pull genes
// from a device work queue in descending-nnz order, or take one fixed gene in the plain
// form. For the gene it computes, for every target g, the exact integers
//     2*U2[g] = sum over target elements x of (2 * #ref{< x} + #ref{== x})  (+ zero block)
//     tie[g]  = sum over distinct values of (t^3 - t) in ref u target g
// and writes U1 = n1*n2 - U2 and the (masked) tie sum; the p-value kernel finishes. This
// reproduces the reference's per-(gene, target) merge (AI4Cell/hpdex
// src/cpp/mannwhitneyu.cpp:618-840, driver :843-1065) without re-walking the reference
// slice for every target: reference ranks come from one bucket index per gene.
//
// Per gene:
//   pass 1  (HBM) 4-wide vector loads of row ids and values; group id gather; value-bucket
//           histograms of all stored elements and of reference elements (bucket = top bits
//           of the key minus the column's minimum key, from the resident matrix's column
//           key ranges); per-group stored counts (and negatives for zero_handling=mix)
//   scan    exclusive prefix sums -> bucket start, reference count below each bucket
//   pass 2  (L2)  scatter (key, group) into bucket order: shared memory when the gene fits,
//           else the CTA's slice of a global scratch buffer (L2-resident)
//   rank    singleton buckets: one atomic; buckets <= kSmallBucket: each element scans its
//           bucket; larger buckets: a warp takes the bucket, extracts its distinct keys in
//           ascending order (repeated warp minimum), and resolves each run of equal keys
//           with per-warp group counters: one representative per (run, target) adds
//           s*(2*lref + c0) and (c0+s)^3-(c0+s)-(c0^3-c0)
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
    const unsigned long long* col_kmin;  // per column min / max key of finite nonzero values
    const unsigned long long* col_kmax;  //   (kmin > kmax: none)
    const unsigned char* col_has_zero;   // per column: stores an explicit finite zero
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
    long long slice;
    unsigned char* acc_global; // per CTA 24*G bytes when the accumulators are not in SMEM
    uint32_t* cnt_global;      // per CTA tie_warps * G counters when not in SMEM
    int32_t nb_max_log2;       // bucket table capacity (power of two)
    int32_t elem_smem_cap;     // elements that fit in shared memory
    int32_t acc_in_smem;
    int32_t cnt_in_smem;
    int32_t tie_warps;         // warps that resolve large buckets (each owns counters)
};

constexpr int kSmallBucket = 8;
constexpr int kMaxRunsByMin = 24;  // distinct keys extracted by warp minimum per bucket

// Shared-memory layout shared by host (sizing) and device (carving).
struct RankSmem {
    size_t hist_bytes, acc_bytes, cnt_bytes, elem_bytes, total;
    __host__ __device__ static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
    __host__ __device__ static int cnt_words(int G) { return G; }
    __host__ __device__ RankSmem(int nb_max_log2, int G, int tie_warps, int acc_in_smem,
                                 int cnt_in_smem, int elem_cap, int key_bytes) {
        const size_t NB = size_t(1) << nb_max_log2;
        hist_bytes = align16((3 * NB + 2) * 4);
        acc_bytes = acc_in_smem ? align16(size_t(G) * 24) : 0;
        cnt_bytes = cnt_in_smem ? align16(size_t(tie_warps) * cnt_words(G) * 4) : 0;
        elem_bytes = align16(size_t(elem_cap) * (key_bytes + 4));
        total = hist_bytes + acc_bytes + cnt_bytes + elem_bytes;
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

// 4 consecutive values starting at a 4-element-aligned position, one or two vector loads
template <class V>
__device__ __forceinline__ void load4(const V* p, V (&v)[4]) {
    if constexpr (sizeof(V) == 4) {
        const uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
        v[0] = __builtin_bit_cast(V, u.x); v[1] = __builtin_bit_cast(V, u.y);
        v[2] = __builtin_bit_cast(V, u.z); v[3] = __builtin_bit_cast(V, u.w);
    } else if constexpr (sizeof(V) == 8) {
        const ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2*>(p));
        const ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2*>(p) + 1);
        v[0] = __builtin_bit_cast(V, a.x); v[1] = __builtin_bit_cast(V, a.y);
        v[2] = __builtin_bit_cast(V, b.x); v[3] = __builtin_bit_cast(V, b.y);
    } else if constexpr (sizeof(V) == 2) {
        const uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
        v[0] = __builtin_bit_cast(V, (uint16_t)(u.x & 0xffffu));
        v[1] = __builtin_bit_cast(V, (uint16_t)(u.x >> 16));
        v[2] = __builtin_bit_cast(V, (uint16_t)(u.y & 0xffffu));
        v[3] = __builtin_bit_cast(V, (uint16_t)(u.y >> 16));
    } else {
        const uint32_t u = __ldg(reinterpret_cast<const uint32_t*>(p));
        v[0] = __builtin_bit_cast(V, (uint8_t)(u & 0xffu));
        v[1] = __builtin_bit_cast(V, (uint8_t)((u >> 8) & 0xffu));
        v[2] = __builtin_bit_cast(V, (uint8_t)((u >> 16) & 0xffu));
        v[3] = __builtin_bit_cast(V, (uint8_t)(u >> 24));
    }
}

// Visits every (row, value) of [p0, p1) once: scalar head and tail, 4-wide aligned body,
// two vectors per thread per iteration so that several loads and gathers are in flight.
template <int NT, class V, class F>
__device__ __forceinline__ void for_each_entry(const int32_t* rows, const V* data, long long p0,
                                               long long p1, F&& f) {
    const int tid = threadIdx.x;
    long long a = (p0 + 3) & ~3ll;
    if (a > p1) a = p1;
    const long long b = a + ((p1 - a) & ~3ll);
    for (long long p = p0 + tid; p < a; p += NT) f(rows[p], data[p]);
    for (long long q = a + 4ll * tid; q < b; q += 8ll * NT) {
        const long long q2 = q + 4ll * NT;
        int4 r0 = __ldg(reinterpret_cast<const int4*>(rows + q));
        V v0[4];
        load4<V>(data + q, v0);
        int4 r1 = make_int4(-1, -1, -1, -1);
        V v1[4] = {V(0), V(0), V(0), V(0)};
        const bool second = q2 < b;
        if (second) {
            r1 = __ldg(reinterpret_cast<const int4*>(rows + q2));
            load4<V>(data + q2, v1);
        }
        f(r0.x, v0[0]); f(r0.y, v0[1]); f(r0.z, v0[2]); f(r0.w, v0[3]);
        if (second) { f(r1.x, v1[0]); f(r1.y, v1[1]); f(r1.z, v1[2]); f(r1.w, v1[3]); }
    }
    for (long long p = b + tid; p < p1; p += NT) f(rows[p], data[p]);
}

// per-warp, per-group counters of a run
__device__ __forceinline__ void cnt_inc(uint32_t* cnt, uint32_t g) { atomicAdd(&cnt[g], 1u); }
__device__ __forceinline__ uint32_t cnt_take(uint32_t* cnt, uint32_t g) {
    // returns the count and clears it; only the first caller per group sees it nonzero
    return atomicExch(&cnt[g], 0u);
}

constexpr uint32_t kRetired = 0xffffffffu;  // group id of an element already resolved

__device__ __forceinline__ unsigned long long tie_delta(unsigned long long c0,
                                                       unsigned long long s) {
    // (c0+s)^3 - (c0+s) - (c0^3 - c0)
    return 3ull * c0 * c0 * s + 3ull * c0 * s * s + s * s * s - s;
}

// Resolves one run of equal keys inside a bucket: the live elements of [s0, s0+m) whose key
// equals `key` (all of them when `pure`). lref = reference elements below the run, c0 =
// reference elements in the run.
template <class K>
__device__ __forceinline__ void resolve_run(const K* ek, const uint32_t* eg, uint32_t s0, uint32_t m,
                                            bool pure, K key, unsigned long long lref,
                                            unsigned long long c0, unsigned long long* A,
                                            unsigned long long* B, uint32_t* cnt,
                                            unsigned long long& tref) {
    const int lane = threadIdx.x & 31;
    for (uint32_t j = lane; j < m; j += 32) {
        const uint32_t g = eg[s0 + j];
        if (g && g != kRetired && (pure || ek[s0 + j] == key)) cnt_inc(cnt, g);
    }
    __syncwarp();
    const unsigned long long a = 2ull * lref + c0;
    for (uint32_t j = lane; j < m; j += 32) {
        const uint32_t g = eg[s0 + j];
        if (g && g != kRetired && (pure || ek[s0 + j] == key)) {
            const unsigned long long s = cnt_take(cnt, g);
            if (s) {
                atomicAdd(&A[g], s * a);
                const unsigned long long tb = tie_delta(c0, s);
                if (tb) atomicAdd(&B[g], tb);
            }
        }
    }
    __syncwarp();
    if (lane == 0) tref += c0 * c0 * c0 - c0;
}

// Warp-level handling of a bucket with more than kSmallBucket elements.
template <class K>
__device__ void resolve_big_bucket(uint32_t b, const uint32_t* hall, const uint32_t* href,
                                   const K* ek, uint32_t* eg, unsigned long long* A,
                                   unsigned long long* B, uint32_t* cnt,
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
    if (lo == hi) {  // pure bucket: a single run
        resolve_run<K>(ek, eg, s0, m, true, lo, rb, c0b, A, B, cnt, tref);
        return;
    }
    // impure: distinct keys in ascending order by repeated warp minimum; resolved elements
    // are retired through their group id (the bucket's slice is private to this warp)
    unsigned long long lref = rb;
    K cur = lo;
    for (int it = 0;; ++it) {
        uint32_t c0 = 0;  // reference elements in the current run
        for (uint32_t j = lane; j < m; j += 32) c0 += (eg[s0 + j] == 0u && ek[s0 + j] == cur);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) c0 += __shfl_xor_sync(0xffffffffu, c0, d);
        resolve_run<K>(ek, eg, s0, m, false, cur, lref, c0, A, B, cnt, tref);
        lref += c0;
        // retire the run and find the next key
        K nxt = ~K(0);
        bool any = false;
        for (uint32_t j = lane; j < m; j += 32) {
            const uint32_t g = eg[s0 + j];
            if (g == kRetired) continue;
            const K k = ek[s0 + j];
            if (k == cur) { eg[s0 + j] = kRetired; continue; }
            nxt = k < nxt ? k : nxt;
            any = true;
        }
        nxt = warp_min(nxt);
        any = __any_sync(0xffffffffu, any);
        __syncwarp();
        if (!any) break;
        if (it + 1 >= kMaxRunsByMin) {
            // many distinct keys (continuous data): finish by brute force per element
            for (uint32_t i = lane; i < m; i += 32) {
                const uint32_t g = eg[s0 + i];
                if (g == kRetired) continue;
                const K k = ek[s0 + i];
                uint32_t lt = 0, e0 = 0, s = 0;
                for (uint32_t j = 0; j < m; ++j) {
                    const uint32_t gj = eg[s0 + j];
                    if (gj == kRetired) continue;
                    const K kj = ek[s0 + j];
                    if (gj == 0u) { lt += (kj < k); e0 += (kj == k); }
                    s += (gj == g && kj == k);
                }
                if (g) {
                    atomicAdd(&A[g], 2ull * (lref + lt) + e0);
                    const unsigned long long cc = e0, ss = s;
                    const unsigned long long tb = 3ull * cc * cc + 3ull * cc * ss + ss * ss - 1ull;
                    if (tb) atomicAdd(&B[g], tb);
                } else {
                    tref += (unsigned long long)e0 * e0 - 1ull;
                }
            }
            __syncwarp();
            break;
        }
        cur = nxt;
    }
}

template <class V, int NT>
__global__ void __launch_bounds__(NT, 1) mwu_rank_kernel(const RankArgs a) {
    using K = typename Val<V>::Key;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_gene;
    __shared__ unsigned long long s_tref;
    __shared__ uint32_t s_nbig;
    __shared__ uint32_t s_wsx[32], s_wsy[32];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int G = a.G, zh = a.zero_handling;
    const int NBMAX = 1 << a.nb_max_log2;
    const RankSmem L(a.nb_max_log2, G, a.tie_warps, a.acc_in_smem, a.cnt_in_smem,
                     a.elem_smem_cap, (int)sizeof(K));
    const int cw = RankSmem::cnt_words(G);

    uint32_t* hall = reinterpret_cast<uint32_t*>(smem);
    uint32_t* href = hall + NBMAX + 1;
    uint32_t* cursor = href + NBMAX + 1;
    unsigned char* accb = a.acc_in_smem ? smem + L.hist_bytes
                                        : a.acc_global + (size_t)blockIdx.x * 24 * G;
    unsigned long long* A = reinterpret_cast<unsigned long long*>(accb);
    unsigned long long* B = A + G;
    uint32_t* nz = reinterpret_cast<uint32_t*>(B + G);
    uint32_t* ng = nz + G;
    uint32_t* cnt_base = a.cnt_in_smem
                             ? reinterpret_cast<uint32_t*>(smem + L.hist_bytes + L.acc_bytes)
                             : a.cnt_global + (size_t)blockIdx.x * a.tie_warps * cw;
    K* ek_s = reinterpret_cast<K*>(smem + L.hist_bytes + L.acc_bytes + L.cnt_bytes);
    uint32_t* eg_s = reinterpret_cast<uint32_t*>(ek_s + a.elem_smem_cap);
    K* ek_g = reinterpret_cast<K*>(a.ek_global) + (size_t)blockIdx.x * a.slice;
    uint32_t* eg_g = a.eg_global + (size_t)blockIdx.x * a.slice;

    const V* data = reinterpret_cast<const V*>(a.data);
    const int32_t* rows = a.rows;
    const int32_t* gidp = a.gid;
    const long long nrows = a.n_rows;

    for (int i = tid; i < a.tie_warps * cw; i += NT) cnt_base[i] = 0u;

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
            s_tref = 0ull;
            s_nbig = 0u;
        }
        first = false;
        for (int g = tid; g < G; g += NT) { A[g] = 0ull; B[g] = 0ull; nz[g] = 0u; ng[g] = 0u; }
        __syncthreads();
        const int c = s_gene;
        if (c < 0) break;
        const long long p0 = a.indptr[c], p1 = a.indptr[c + 1];

        // ---- bucket function from the column's key range ----
        K kmin = (K)a.col_kmin[c], kmax = (K)a.col_kmax[c];
        if (zh == ZH_NONE && a.col_has_zero[c]) {
            const K kz = Val<V>::key(V(0));
            kmin = kz < kmin ? kz : kmin;
            kmax = kz > kmax ? kz : kmax;
        }
        const long long nraw = p1 - p0;
        int nbl = 1;
        while (nbl < a.nb_max_log2 && (1ll << nbl) < 2 * nraw) ++nbl;
        const int NB = 1 << nbl;
        int shift = 0;
        if (kmin <= kmax) {
            const int bl = bit_length(K(kmax - kmin));
            shift = bl > nbl ? bl - nbl : 0;
        }
        for (int b = tid; b <= NB; b += NT) { hall[b] = 0u; href[b] = 0u; }
        __syncthreads();

        // ---- pass 1: histograms and per-group stored counts ----
        uint32_t nref_local = 0;
        for_each_entry<NT, V>(rows, data, p0, p1, [&](int32_t r, V v) {
            if (r < 0 || (long long)r >= nrows) return;
            const int g = __ldg(gidp + r);
            if (g < 0 || g >= G) return;
            if (!Val<V>::finite(v)) return;
            if (zh != ZH_NONE && Val<V>::zero(v)) return;
            if (g) atomicAdd(&nz[g], 1u);
            else ++nref_local;
            if (zh == ZH_MIX && Val<V>::neg(v)) atomicAdd(&ng[g], 1u);
            const uint32_t b = (uint32_t)((Val<V>::key(v) - kmin) >> shift);
            atomicAdd(&hall[b], 1u);
            if (g == 0) atomicAdd(&href[b], 1u);
        });
        for (int d = 16; d > 0; d >>= 1) nref_local += __shfl_xor_sync(0xffffffffu, nref_local, d);
        if (lane == 0 && nref_local) atomicAdd(&nz[0], nref_local);
        __syncthreads();
        block_scan2<NT>(hall, href, NB, s_wsx, s_wsy);
        const uint32_t n = hall[NB];
        for (int b = tid; b < NB; b += NT) cursor[b] = hall[b];
        const bool in_smem = n <= (uint32_t)a.elem_smem_cap;
        K* ek = in_smem ? ek_s : ek_g;
        uint32_t* eg = in_smem ? eg_s : eg_g;
        __syncthreads();

        // ---- pass 2: scatter into bucket order ----
        for_each_entry<NT, V>(rows, data, p0, p1, [&](int32_t r, V v) {
            if (r < 0 || (long long)r >= nrows) return;
            const int g = __ldg(gidp + r);
            if (g < 0 || g >= G) return;
            if (!Val<V>::finite(v)) return;
            if (zh != ZH_NONE && Val<V>::zero(v)) return;
            const K k = Val<V>::key(v);
            const uint32_t b = (uint32_t)((k - kmin) >> shift);
            const uint32_t pos = atomicAdd(&cursor[b], 1u);
            ek[pos] = k;
            eg[pos] = (uint32_t)g;
        });
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
                    const unsigned long long cc = c0, ss = s;
                    const unsigned long long tb = 3ull * cc * cc + 3ull * cc * ss + ss * ss - 1ull;
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
            uint32_t* cnt = cnt_base + (size_t)warp * cw;
            const uint32_t nbig = s_nbig;
            for (uint32_t q = warp; q < nbig; q += a.tie_warps)
                resolve_big_bucket<K>(cursor[q], hall, href, ek, eg, A, B, cnt, tref);
        }
        tref = warp_sum_u64(tref);
        if (lane == 0 && tref) atomicAdd(&s_tref, tref);
        __syncthreads();

        // ---- finalize per target ----
        const unsigned long long T_ref = s_tref;
        const unsigned long long nz1 = nz[0];
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
        __syncthreads();
    }
}

// Per-column key range of finite nonzero values and whether an explicit finite zero is
// stored; computed once when a matrix becomes resident (one warp per column).
template <class V>
__global__ void column_key_range_kernel(const V* data, const int64_t* indptr, int32_t n_cols,
                                        unsigned long long* kmin, unsigned long long* kmax,
                                        unsigned char* has_zero) {
    using K = typename Val<V>::Key;
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int c = blockIdx.x * wpb + (threadIdx.x >> 5); c < n_cols; c += gridDim.x * wpb) {
        K lo = ~K(0), hi = K(0);
        bool z = false;
        for (long long p = indptr[c] + lane; p < indptr[c + 1]; p += 32) {
            const V v = data[p];
            if (!Val<V>::finite(v)) continue;
            if (Val<V>::zero(v)) { z = true; continue; }
            const K k = Val<V>::key(v);
            lo = k < lo ? k : lo;
            hi = k > hi ? k : hi;
        }
        lo = warp_min(lo);
        hi = warp_max(hi);
        z = __any_sync(0xffffffffu, z);
        if (lane == 0) {
            kmin[c] = lo;
            kmax[c] = hi;
            has_zero[c] = z ? 1 : 0;
        }
    }
}

}  // namespace hpdex
