// mwu_rank.cuh -- per-gene rank-sum kernel of the Mann-Whitney U backend (sm_103a).
//
// One CTA owns one gene (CSC column) at a time; persistent CTAs (one per SM) pull genes
// from a device work queue in descending-nnz order, or take one fixed gene in the plain
// form. For the gene it computes, for every target g, the exact integers
//     2*U2[g] = sum over target elements x of (2 * #ref{< x} + #ref{== x})  (+ zero block)
//     tie[g]  = sum over distinct values of (t^3 - t) in ref u target g
// and writes U1 = n1*n2 - U2 and the (masked) tie sum; a p-value kernel finishes, or the
// kernel computes the p-values itself during the next gene (fused p-values, below). This
// reproduces the reference's per-(gene, target) merge (AI4Cell/hpdex
// src/cpp/mannwhitneyu.cpp:618-840, driver :843-1065) without re-walking the reference
// slice for every target: reference ranks come from one bucket index per gene.
//
// Per gene:
//   pass 1  (HBM, evict-first loads) warp tiles of 128 entries, 4 per lane with neighbouring
//           lanes on neighbouring entries: row ids and values, group id gathers, decode to
//           (key, group) written at the entry's position in the CTA's
//           scratch slice; value-bucket histograms of all stored elements and of reference
//           elements (bucket = top bits of key - column minimum key, from the resident
//           matrix's column key ranges); per-group stored counts (negatives for mix)
//   scan    exclusive prefix sums -> bucket start, reference count below each bucket
//   slabs   the whole gene when it fits in shared memory, else consecutive bucket ranges
//           holding at most the shared-memory element capacity; per slab:
//   pass 2  (L2) scatter the slab's decoded elements into bucket order in shared memory (a
//           slab made of one bucket larger than half the capacity uses a global slice);
//           after the last slab the decoded copy is dropped from L2 without write-back
//           (discard.global.L2)
//   rank    32-bucket chunks to all warps: singleton buckets add one term; buckets of 2..32
//           elements are packed whole into 32-lane warp rounds: reference
//           lanes are broadcast to count smaller / equal reference keys, per-warp group
//           counters find repeated (key, group) pairs; larger buckets go to a list that
//           warps drain one bucket at a time with per-warp group counters: one
//           representative per (run of equal keys, target) adds s*(2*lref + c0) to A and
//           (c0+s)^3-(c0+s)-(c0^3-c0) to B
//   final   zero block, U1, tie sum per target (fused: P during the next gene's rank phase);
//           the gene clears the bucket-table entries it used, and one thread fetches the
//           next gene and its column metadata
//
// Shared-memory accumulators use 32-bit atomics (a 64-bit value is updated as two halves
// with an explicit carry): on sm_103a a 64-bit shared atomic add costs about five times a
// 32-bit one, and warp match instructions about six ballots, so neither is used per round.
//
// "Stored" elements are what the reference gathers into its slices (mannwhitneyu.cpp:
// 914-926): row id in [0, n_rows), group in [0, G), finite value; for zero_handling
// min/max/mix explicit zeros are left out too and join the implicit-zero block, whose size
// per group is group_rows[g] - stored[g] (:967-1003).
#pragma once
#include <climits>
#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "pvalue_math.cuh"

namespace hpdex {

constexpr int kErrWords = 2;  // error words of a run, reset to all ones before it

// One task = one (resident matrix, grouping) pair with its outputs. A launch ranks the genes
// of one task, or of several (the serving loop coalesces queries into one launch); the tasks
// of a launch share the value type and the shared-memory layout (sized for the largest G).
struct RankTask {
    const void* data;          // values of the CSC matrix (dtype V)
    const int32_t* rows;       // row ids (int32)
    const int64_t* indptr;     // [n_cols + 1]
    const unsigned long long* col_kmin;  // per column min / max key of finite nonzero values
    const unsigned long long* col_kmax;  //   (kmin > kmax: none)
    const uint32_t* col_has_zero;        // per column: bit 0 stores an explicit finite zero,
                                         // bit 1 stores a finite value that is not an integer
                                         // of magnitude below 2^31 (no histogram path)
    int64_t n_rows;
    int32_t n_cols;
    int32_t G;                 // n_targets + 1 (at most the launch's layout G)
    const void* group_of_row;  // [n_rows] group of each row in the kernel's group type
                               // (GroupType below), all ones for rows in no group
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
    // p-value options, used when the launch computes p-values (RankArgs::erfc_table)
    int32_t alternative;
    int32_t fast_norm;
    double cc;                 // continuity correction (0.5 or 0)
    const PConst* pconst;      // zero_handling min / max / mix: per target (or null)
    int32_t compact_decode;    // 1: the decoded copy keeps stored entries only (set when the
                               // grouping leaves many rows out: fewer entries to re-read)
};

struct RankArgs {
    const RankTask* tasks;     // device array of the launch's tasks
    const int32_t* order;      // genes in processing order [n_order]
    const uint16_t* order_task;  // task of each entry of `order` (null: all task 0)
    int32_t n_order;
    int32_t* queue;            // work counter (batched form)
    int32_t single_gene;       // >= 0: plain form, this gene of task 0 only
    int32_t G;                 // layout G: the largest task G of the launch
    // global scratch, one slice of `slice` elements per CTA for each of:
    void* dk_global;           // decoded keys of the current gene, at the entries' positions
    void* dg_global;           // decoded groups (group type; all ones: not stored)
    void* ek_global;           // bucket-ordered elements of a slab too big for shared memory
    void* eg_global;
    long long slice;           // rank_slice(longest column of any task): multiple of 64
    unsigned char* acc_global; // per CTA 24*G bytes when the accumulators are not in SMEM
    uint32_t* cnt_global;      // per CTA and warp: packed counters (when not in SMEM), then
                               // G 32-bit counters (buckets of more than 65535 elements)
    int32_t nb_max_log2;       // bucket table capacity (power of two, at most 2^13: the scan
                               // holds 8 entries per thread)
    int32_t elem_smem_cap;     // elements that fit in shared memory
    int32_t acc_in_smem;       // accumulators and packed run counters in shared memory
    int32_t cnt_in_smem;       // run counters in shared memory (with the accumulators; else in
                               // global memory, and rounds resolve repeated groups by warp match)
    int32_t tie_warps;         // = warps per CTA (each owns packed run counters)
    const double* erfc_table;  // non-null: the kernel also computes the asymptotic p-values
                               // (P replaces the tie sums); null: a p-value kernel follows
    int32_t drain_wait;        // 1: a warp that finds a big-list entry not yet published polls
                               // for it a bounded number of times; 0 (the default): it goes to
                               // the block barrier at once (the results are the same)
    int32_t no_histogram;      // 1: every gene takes the bucket path, and the launch uses the
                               // kernel without the histogram path; 0: the histogram path is
                               // chosen per gene (hist_choice)
    int32_t any_compact;       // some task has compact_decode set (the launch uses the kernel
                               // variant that can compact)
    int32_t cta_base;          // per-CTA scratch slice of CTA b: cta_base + b (the plain form
                               // runs one-CTA launches on concurrent streams, each on its slice)
};

constexpr int kMediumBucket = 32;  // 2..32: packed whole into warp rounds
constexpr int kMaxRunsByMin = 24;  // distinct keys extracted by warp minimum per bucket
constexpr uint32_t kInvalid = 0xffffffffu;
constexpr uint32_t kTaken = 0xfffffffeu;    // a big-list entry that a warp has resolved
constexpr int kDrainWaitIters = 4096;       // polls (with a short sleep) for a big-list entry
constexpr int kPvWarps = 4;                 // warps (one per SM sub-partition) that take a
                                            // gene's p-value tiles at the start of the next
                                            // gene's rank phase; warps waiting in its drain
                                            // take further tiles
// Group ids inside the kernel: 16-bit when the accumulators are in shared memory (which
// bounds G far below 65535), else 32-bit; all ones marks an entry outside every group.
template <bool ACC_SMEM>
using GroupType = std::conditional_t<ACC_SMEM, uint16_t, uint32_t>;
__host__ __device__ inline int group_bytes(int acc_in_smem) { return acc_in_smem ? 2 : 4; }

// Scratch slice per CTA: the longest column in whole 128-byte lines of 16-bit elements
// (discard.global.L2 works on lines, so no line of a slice is shared with another CTA's).
__host__ __device__ inline long long rank_slice(long long longest) {
    return ((longest > 0 ? longest : 1) + 63) & ~63ll;
}

// Shared-memory layout shared by host (sizing) and device (carving): accumulators, run
// counters, then bucket starts and reference counts (NB + 1 each, padded to 16 bytes) with the
// slab's list of large buckets, then elements. The last two are contiguous: a gene on the
// histogram path uses both as its (value, group) counters.
struct RankSmem {
    size_t hist_bytes, acc_bytes, cnt_bytes, elem_bytes, total;
    __host__ __device__ static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
    __host__ __device__ static int cnt_words(int G) { return (G + 1) / 2; }
    // elements the element region holds with 16-bit key offsets (compact slabs)
    __host__ __device__ static int compact_cap(int elem_cap, int key_bytes, int acc_in_smem) {
        const int gb = group_bytes(acc_in_smem);
        return (int)(((long long)elem_cap * (key_bytes + gb) / (2 + gb)) & ~7ll);
    }
    // a slab holds at most (compact) capacity elements outside one oversized bucket, so it has
    // at most capacity / (kMediumBucket + 1) + 2 buckets above kMediumBucket
    __host__ __device__ static int big_list(int max_elems) { return max_elems / 33 + 64; }
    __host__ __device__ RankSmem(int nb_max_log2, int G, int tie_warps, int acc_in_smem,
                                 int cnt_in_smem, int elem_cap, int key_bytes) {
        const size_t NB = size_t(1) << nb_max_log2;
        hist_bytes = align16((2 * (NB + 4) + big_list(compact_cap(elem_cap, key_bytes, acc_in_smem))) * 4);
        acc_bytes = acc_in_smem ? align16(size_t(G) * 24) : 0;
        cnt_bytes = cnt_in_smem ? align16(size_t(tie_warps) * cnt_words(G) * 4) : 0;
        elem_bytes = align16(size_t(elem_cap) * (key_bytes + group_bytes(acc_in_smem)));
        total = hist_bytes + acc_bytes + cnt_bytes + elem_bytes;
    }
};

// ---------------------------------------------------------------------------------------
// Atomics. SH = the address is in shared memory: explicit .shared forms, so that a pointer
// that reaches a helper as a generic pointer still compiles to a shared-memory atomic.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
template <bool SH>
__device__ __forceinline__ void red_add(uint32_t* p, uint32_t v) {
    if constexpr (SH) asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(smem_addr(p)), "r"(v) : "memory");
    else atomicAdd(p, v);
}
template <bool SH>
__device__ __forceinline__ uint32_t atom_add(uint32_t* p, uint32_t v) {
    if constexpr (SH) {
        uint32_t o;
        asm volatile("atom.shared.add.u32 %0, [%1], %2;" : "=r"(o) : "r"(smem_addr(p)), "r"(v) : "memory");
        return o;
    } else {
        return atomicAdd(p, v);
    }
}
template <bool SH>
__device__ __forceinline__ uint32_t atom_and(uint32_t* p, uint32_t v) {
    if constexpr (SH) {
        uint32_t o;
        asm volatile("atom.shared.and.b32 %0, [%1], %2;" : "=r"(o) : "r"(smem_addr(p)), "r"(v) : "memory");
        return o;
    } else {
        return atomicAnd(p, v);
    }
}
// 64-bit accumulator update: in shared memory a 32-bit add to the low half whose wrap-around
// (seen in the value the atomic returns) carries into the high half; the halves are only
// read as one 64-bit value after a block barrier. Global memory: native 64-bit atomics.
template <bool SH>
__device__ __forceinline__ void acc_add(unsigned long long* p, unsigned long long v) {
    if constexpr (SH) {
        uint32_t* w = reinterpret_cast<uint32_t*>(p);
        const uint32_t lo = (uint32_t)v;
        uint32_t hi = (uint32_t)(v >> 32);
        if (lo) {
            const uint32_t old = atom_add<true>(w, lo);
            hi += (uint32_t)(old + lo < old);
        }
        if (hi) red_add<true>(w + 1, hi);
    } else {
        if (v) atomicAdd(p, v);
    }
}

// Drops the 128-byte L2 lines of [p, p + bytes) without write-back (p 128-byte aligned; the
// lines belong to this CTA's scratch slice and hold nothing that is read again).
template <int NT>
__device__ __forceinline__ void l2_discard(const void* p, size_t bytes) {
    const char* b = static_cast<const char*>(p);
    for (size_t o = (size_t)threadIdx.x * 128; o < bytes; o += (size_t)NT * 128)
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(b + o) : "memory");
}

template <int NT>
__device__ void block_scan2(uint32_t* x, uint32_t* y, int L, uint32_t* wsx, uint32_t* wsy,
                            uint32_t* xmax) {
    // exclusive prefix sums of x[0..L) and y[0..L) in place; x[L], y[L] = totals;
    // *xmax = max x[i] (the caller zeroes it before). x and y are 16-byte aligned; a thread
    // owns `per` consecutive entries, moved with 128-bit accesses when per is 4 or 8.
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (L + NT - 1) / NT;
    const int beg = min(L, tid * per), cnt = min(L, beg + per) - beg;
    uint32_t vx[8], vy[8];
    if (cnt == 8 || cnt == 4) {
        const uint4 a0 = *reinterpret_cast<const uint4*>(x + beg);
        const uint4 b0 = *reinterpret_cast<const uint4*>(y + beg);
        vx[0] = a0.x; vx[1] = a0.y; vx[2] = a0.z; vx[3] = a0.w;
        vy[0] = b0.x; vy[1] = b0.y; vy[2] = b0.z; vy[3] = b0.w;
        if (cnt == 8) {
            const uint4 a1 = *reinterpret_cast<const uint4*>(x + beg + 4);
            const uint4 b1 = *reinterpret_cast<const uint4*>(y + beg + 4);
            vx[4] = a1.x; vx[5] = a1.y; vx[6] = a1.z; vx[7] = a1.w;
            vy[4] = b1.x; vy[5] = b1.y; vy[6] = b1.z; vy[7] = b1.w;
        } else {
#pragma unroll
            for (int i = 4; i < 8; ++i) { vx[i] = 0u; vy[i] = 0u; }
        }
    } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            vx[i] = i < cnt ? x[beg + i] : 0u;
            vy[i] = i < cnt ? y[beg + i] : 0u;
        }
    }
    uint32_t sx = 0, sy = 0, mx = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) { sx += vx[i]; sy += vy[i]; mx = max(mx, vx[i]); }
    mx = __reduce_max_sync(0xffffffffu, mx);
    if (lane == 0 && mx) atomicMax(xmax, mx);
    const uint32_t ix = warp_incl_scan(sx), iy = warp_incl_scan(sy);
    if (lane == 31) { wsx[warp] = ix; wsy[warp] = iy; }
    __syncthreads();
    // every warp scans the warp totals itself (no second barrier)
    uint32_t ox, oy;
    {
        const uint32_t ux = lane < NT / 32 ? wsx[lane] : 0u;
        const uint32_t uy = lane < NT / 32 ? wsy[lane] : 0u;
        const uint32_t px = warp_incl_scan(ux), py = warp_incl_scan(uy);
        ox = __shfl_sync(0xffffffffu, px - ux, warp) + ix - sx;
        oy = __shfl_sync(0xffffffffu, py - uy, warp) + iy - sy;
        if (warp == 0 && lane == 31) { x[L] = px; y[L] = py; }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t tx = vx[i], ty = vy[i];
        vx[i] = ox; ox += tx;
        vy[i] = oy; oy += ty;
    }
    if (cnt == 8 || cnt == 4) {
        *reinterpret_cast<uint4*>(x + beg) = make_uint4(vx[0], vx[1], vx[2], vx[3]);
        *reinterpret_cast<uint4*>(y + beg) = make_uint4(vy[0], vy[1], vy[2], vy[3]);
        if (cnt == 8) {
            *reinterpret_cast<uint4*>(x + beg + 4) = make_uint4(vx[4], vx[5], vx[6], vx[7]);
            *reinterpret_cast<uint4*>(y + beg + 4) = make_uint4(vy[4], vy[5], vy[6], vy[7]);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if (i < cnt) { x[beg + i] = vx[i]; y[beg + i] = vy[i]; }
    }
    __syncthreads();
}

// Streaming (evict-first) loads of the matrix: each entry is read once per run.
template <class V>
__device__ __forceinline__ V ld_stream(const V* p) {
    if constexpr (sizeof(V) == 8) return __builtin_bit_cast(V, __ldcs(reinterpret_cast<const unsigned long long*>(p)));
    else if constexpr (sizeof(V) == 4) return __builtin_bit_cast(V, __ldcs(reinterpret_cast<const unsigned int*>(p)));
    else if constexpr (sizeof(V) == 2) return __builtin_bit_cast(V, __ldcs(reinterpret_cast<const unsigned short*>(p)));
    else return __builtin_bit_cast(V, __ldcs(reinterpret_cast<const unsigned char*>(p)));
}
// Per-warp, per-group counters of a run, 16 bits each (two groups per 32-bit word). A run
// never counts more than 65535 elements of one group here: buckets with more than 65535
// elements are resolved with 32-bit counters instead.
template <bool SH>
__device__ __forceinline__ void cnt_inc(uint32_t* cnt, uint32_t g) {
    red_add<SH>(&cnt[g >> 1], (g & 1u) ? 0x10000u : 1u);
}
template <bool SH>
__device__ __forceinline__ uint32_t cnt_take(uint32_t* cnt, uint32_t g) {
    // returns the count and clears it; only the first caller per group sees it nonzero
    const uint32_t old = atom_and<SH>(&cnt[g >> 1], (g & 1u) ? 0x0000ffffu : 0xffff0000u);
    return (g & 1u) ? (old >> 16) : (old & 0xffffu);
}
__device__ __forceinline__ void cntw_inc(uint32_t* cnt, uint32_t g) { atomicAdd(&cnt[g], 1u); }
__device__ __forceinline__ uint32_t cntw_take(uint32_t* cnt, uint32_t g) { return atomicExch(&cnt[g], 0u); }

__device__ __forceinline__ unsigned long long tie_delta(unsigned long long c0,
                                                       unsigned long long s) {
    // (c0+s)^3 - (c0+s) - (c0^3 - c0)
    return 3ull * c0 * c0 * s + 3ull * c0 * s * s + s * s * s - s;
}

template <class K>
__device__ __forceinline__ K wmin(unsigned mask, K v) {
    if constexpr (sizeof(K) == 4) return __reduce_min_sync(mask, v);
    else return warp_min(v);
}
template <class K>
__device__ __forceinline__ K wmax(unsigned mask, K v) {
    if constexpr (sizeof(K) == 4) return __reduce_max_sync(mask, v);
    else return warp_max(v);
}

// Accumulator set of a gene: A (doubled U2 terms) and B (target tie terms) per group.
struct Acc {
    unsigned long long* A;
    unsigned long long* B;
};

// Adds the contribution of s equal (key, target g) elements whose run has c0 reference
// elements and lref reference elements below it.
template <bool SH>
__device__ __forceinline__ void add_pair(const Acc& acc, uint32_t g, unsigned long long s,
                                         unsigned long long lref, unsigned long long c0) {
    acc_add<SH>(&acc.A[g], s * (2ull * lref + c0));
    acc_add<SH>(&acc.B[g], tie_delta(c0, s));
}

// One warp round over up to 32 elements of buckets that lie wholly inside the round:
// lane L holds (key, g) when active; `sub` is the lane mask of L's bucket, rb its reference
// count below. Every element adds its own share, so no representative is needed:
//   target: A += 2*(rb + lt) + c0, B += 3c0^2 + 3c0*s + s^2 - 1
//   reference: T_ref += c0^2 - 1
// where lt / c0 count the reference elements of the bucket with a smaller / equal key and s
// the target elements with the same key and group (keys of different buckets are never
// compared: they may be 16-bit offsets inside their buckets). Summed over a run of c0 reference and
// s target-g elements these give s*(2*lref + c0), (c0+s)^3-(c0+s)-(c0^3-c0) and c0^3-c0.
// Most buckets of a round hold one key (a tie run): there every reference element of the
// bucket is equal (lt = 0, c0 = its reference lanes) and equal groups mean equal (key, group).
// Buckets with more than one key take lt and c0 from broadcasting their (few) reference lanes.
// s: the warp's group counters show which groups occur more than once in the round; such lanes
// of one-key buckets match their group, those of other buckets compare pairwise among
// themselves. `cnt` is zero on entry and on exit. RM (the counters are in global memory, where
// a round's increments, read-back and clear would cost more): one warp match over the target
// lanes' groups instead of the counters.
template <class K, bool SH, bool RM>
__device__ __forceinline__ void resolve_round(bool active, K key, uint32_t g, unsigned sub,
                                              uint32_t rb, const Acc& acc, uint32_t* cnt,
                                              unsigned long long& tref) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!act) return;
    const bool is_ref = active && g == 0u;
    const bool is_tar = active && g != 0u;
    const unsigned refm = __ballot_sync(0xffffffffu, is_ref);
    // buckets with more than one key: some lane's key differs from its bucket's first lane's
    const int first = active ? __ffs((int)sub) - 1 : (int)(threadIdx.x & 31);
    const K kf = __shfl_sync(0xffffffffu, key, first);
    const unsigned diff = __ballot_sync(0xffffffffu, active && key != kf);
    const bool mixed = (sub & diff) != 0u;
    const unsigned mixm = __ballot_sync(0xffffffffu, active && mixed);
    uint32_t lt = 0, c0 = mixed ? 0u : (uint32_t)__popc(refm & sub);
    for (unsigned r = refm & mixm; r; r &= r - 1u) {
        const int j = __ffs((int)r) - 1;
        const K kj = __shfl_sync(0xffffffffu, key, j);
        if ((sub >> j) & 1u) {
            lt += kj < key;
            c0 += kj == key;
        }
    }
    uint32_t s = 1, ng = 0;
    bool repeats = true;  // (warp-uniform) some target group occurs more than once in the round
    if constexpr (RM) {
        // target lanes with this lane's group (other lanes match nobody: group ids are below 2^31)
        const unsigned same = __match_any_sync(0xffffffffu, is_tar ? g : (0x80000000u | (threadIdx.x & 31u)));
        ng = is_tar ? (uint32_t)__popc(same) : 0u;
        if (ng > 1u && !mixed) s = (uint32_t)__popc(same & sub);
    } else {
        if (is_tar) cnt_inc<SH>(cnt, g);
        __syncwarp();
        if (is_tar) {
            const uint32_t w = cnt[g >> 1];
            ng = (g & 1u) ? (w >> 16) : (w & 0xffffu);
        }
        __syncwarp();
        if (is_tar) cnt[g >> 1] = 0u;  // clears both groups of the word; both were read above
        repeats = __ballot_sync(0xffffffffu, ng > 1u) != 0u;
        if (repeats) {
            // every lane of a one-key bucket whose group repeats in the round is in `one`, so
            // the match over `one` sees all lanes of its bucket with its group
            const unsigned one = __ballot_sync(0xffffffffu, ng > 1u && !mixed);
            if (ng > 1u && !mixed) s = (uint32_t)__popc(__match_any_sync(one, g) & sub);
        }
    }
    if (repeats) {
        // lanes of buckets with several keys whose group repeats: every lane with the same
        // bucket, key and group is among them
        const unsigned many = __ballot_sync(0xffffffffu, ng > 1u && mixed);
        if (many) {
            uint32_t c = 0;
            for (unsigned r = many; r; r &= r - 1u) {
                const int j = __ffs((int)r) - 1;
                const K kj = __shfl_sync(0xffffffffu, key, j);
                const uint32_t gj = __shfl_sync(0xffffffffu, g, j);
                c += ((sub >> j) & 1u) && gj == g && kj == key;  // same bucket: keys may be offsets
            }
            if (ng > 1u && mixed) s = c;
        }
    }
    __syncwarp();
    if (is_tar) {
        acc_add<SH>(&acc.A[g], 2ull * ((unsigned long long)rb + lt) + c0);
        const uint32_t tb = 3u * c0 * c0 + 3u * c0 * s + s * s - 1u;  // c0, s <= 32
        if (tb) acc_add<SH>(&acc.B[g], tb);
    } else if (is_ref) {
        tref += (unsigned long long)c0 * c0 - 1ull;
    }
}

// Warp-level resolution of a bucket of more than kMediumBucket elements [s0, s0+m).
// Pass A counts the targets per group assuming the bucket is pure (one key) while finding
// its key range and reference count; pure buckets finish with pass B (one representative
// per group adds the contribution). Impure buckets undo the counts and visit their distinct
// keys in ascending order (warp minimum), two passes per key; after kMaxRunsByMin keys the
// rest is resolved element by element. Counters are zero on entry and on exit.
// SH: accumulators in shared memory; SHC: counters in shared memory.
template <class K, bool WIDE, bool SH, bool SHC, class EK, class EG>
__device__ void resolve_big(uint32_t s0, uint32_t m, uint32_t rb, const EK* ek, const EG* eg,
                            const Acc& acc, uint32_t* cnt, unsigned long long& tref) {
    const int lane = threadIdx.x & 31;
    auto inc = [&](uint32_t g) {
        if constexpr (WIDE) cntw_inc(cnt, g);
        else cnt_inc<SHC>(cnt, g);
    };
    auto take = [&](uint32_t g) -> uint32_t {
        if constexpr (WIDE) return cntw_take(cnt, g);
        else return cnt_take<SHC>(cnt, g);
    };
    K lo = ~K(0), hi = K(0);
    uint32_t c0 = 0;
    for (uint32_t j = lane; j < m; j += 32) {
        const K k = ek[s0 + j];
        const uint32_t g = eg[s0 + j];
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
        if (g) inc(g);
        else ++c0;
    }
    lo = wmin<K>(0xffffffffu, lo);
    hi = wmax<K>(0xffffffffu, hi);
    c0 = __reduce_add_sync(0xffffffffu, c0);
    __syncwarp();
    if (lo == hi) {
        for (uint32_t j = lane; j < m; j += 32) {
            const uint32_t g = eg[s0 + j];
            if (g) {
                const uint32_t s = take(g);
                if (s) add_pair<SH>(acc, g, s, rb, c0);
            }
        }
        if (lane == 0) tref += (unsigned long long)c0 * c0 * c0 - c0;
        __syncwarp();
        return;
    }
    // impure: clear the counts, then one key at a time
    for (uint32_t j = lane; j < m; j += 32) {
        const uint32_t g = eg[s0 + j];
        if (g) (void)take(g);
    }
    __syncwarp();
    unsigned long long lref = rb;
    K cur = lo;
    for (int it = 0;; ++it) {
        uint32_t r0 = 0;
        for (uint32_t j = lane; j < m; j += 32) {
            if (ek[s0 + j] != cur) continue;
            const uint32_t g = eg[s0 + j];
            if (g) inc(g);
            else ++r0;
        }
        r0 = __reduce_add_sync(0xffffffffu, r0);
        __syncwarp();
        K nxt = ~K(0);
        bool more = false;
        for (uint32_t j = lane; j < m; j += 32) {
            const K k = ek[s0 + j];
            if (k == cur) {
                const uint32_t g = eg[s0 + j];
                if (g) {
                    const uint32_t s = take(g);
                    if (s) add_pair<SH>(acc, g, s, lref, r0);
                }
            } else if (k > cur) {
                nxt = k < nxt ? k : nxt;
                more = true;
            }
        }
        if (lane == 0) tref += (unsigned long long)r0 * r0 * r0 - r0;
        lref += r0;
        more = __any_sync(0xffffffffu, more);
        nxt = wmin<K>(0xffffffffu, nxt);
        __syncwarp();
        if (!more) break;
        if (it + 1 >= kMaxRunsByMin) {
            // many distinct keys (continuous data): the elements with key >= nxt one by one
            for (uint32_t i = lane; i < m; i += 32) {
                const K k = ek[s0 + i];
                if (k < nxt) continue;
                const uint32_t g = eg[s0 + i];
                uint32_t lt = 0, e0 = 0, sc = 0;
                for (uint32_t j = 0; j < m; ++j) {
                    const K kj = ek[s0 + j];
                    if (kj < nxt) continue;
                    const uint32_t gj = eg[s0 + j];
                    if (gj == 0u) { lt += (kj < k); e0 += (kj == k); }
                    sc += (gj == g && kj == k);
                }
                if (g) {
                    acc_add<SH>(&acc.A[g], 2ull * (lref + lt) + e0);
                    const unsigned long long cc = e0, ss = sc;
                    acc_add<SH>(&acc.B[g], 3ull * cc * cc + 3ull * cc * ss + ss * ss - 1ull);
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

// ---------------------------------------------------------------------------------------
// Fused p-values. A gene's finalize writes U1 and the tie sum of its tests; the FP64 work of
// turning them into p-values is left pending and done during the next gene's rank phase, by
// kPvWarps warps at its start and by warps that would otherwise wait in its drain, while the
// other warps keep the integer pipes busy (FP64 is the scarce pipe on GB300, and the rank phase
// hardly uses it). Tiles still pending before the finalize are taken by all warps; the CTA's
// last gene is finished by all warps after the work queue runs dry.
// ---------------------------------------------------------------------------------------
// Tests of targets 1 + 32q + lane of gene c: P replaces the tie sum. Not inlined, so that the
// FP64 arithmetic's registers stay out of the rank loops' allocation (one test per lane: more
// independent chains per warp cost the rank loops more than they gain).
static __device__ __noinline__ void pvalue_tile(const RankTask* tk, int c, uint32_t q, const double* tbl) {
    const int g = 1 + 32 * (int)q + (int)(threadIdx.x & 31);
    if (g >= tk->G) return;
    const size_t idx = (size_t)(g - 1) * tk->n_cols + c;
    double n1, n2;
    if (tk->zero_handling == ZH_NONE) {
        n1 = (double)tk->n1[c];
        n2 = (double)tk->n2[idx];
    } else {
        n1 = (double)tk->group_rows[0];
        n2 = (double)tk->group_rows[g];
    }
    const double u1 = tk->U1[idx], ts = tk->tie[idx];
    double p;
    if (tk->fast_norm) p = p_asymptotic_fast(u1, n1, n2, ts, tk->cc, tk->alternative);
    else if (tk->pconst && tk->zero_handling != ZH_NONE)
        p = p_asymptotic_k(u1, tk->pconst[g - 1], ts, tk->cc, tk->alternative, tbl);
    else p = p_asymptotic(u1, n1, n2, ts, tk->cc, tk->alternative, tbl);
    tk->tie[idx] = p;
}

// The calling warp takes tiles of 32 tests of gene c until none is left (*s_pvq counts the
// tiles taken).
__device__ __forceinline__ void pvalue_tiles(const RankTask* tk, int c, uint32_t* s_pvq,
                                             const double* tbl) {
    const uint32_t ntiles = ((uint32_t)tk->G + 30u) / 32u;  // ceil((G - 1) / 32)
    for (;;) {
        uint32_t q = 0;
        if ((threadIdx.x & 31) == 0) q = atomicAdd(s_pvq, 1u);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= ntiles) break;
        pvalue_tile(tk, c, q, tbl);
    }
}

// Rank phase of one slab: elements [0, cnt) in bucket order in ek/eg, buckets [blo, bhi)
// starting at `base` in the gene's bucket order (hall[b - 1] = start of bucket b).
// Buckets of 2..32 elements are packed whole, in bucket order, into rounds of up to 32
// lanes; `tbl` (32 bytes per warp) maps the k-th such bucket of a chunk to its lane.
// RM: the run counters are in global memory (rounds by warp match, see resolve_round).
template <class K, bool SH, bool RM, class EK, class EG>
__device__ void rank_slab(const EK* ek, const EG* eg, uint32_t blo, uint32_t bhi, uint32_t base,
                          const uint32_t* hall, const uint32_t* href, uint32_t* biglist,
                          uint32_t biglist_cap, uint32_t* s_chunk, uint32_t* s_nbig,
                          uint32_t* s_bigi, uint32_t* s_wdone, const Acc& acc, uint32_t* cnt,
                          uint32_t* wide_cnt, uint8_t* tbl, unsigned long long& tref,
                          const RankTask* pv_tk, int pv_c, uint32_t* s_pvq, const double* erfc_table,
                          int wait_polls) {
    const int lane = threadIdx.x & 31;
    const uint32_t nchunks = (bhi - blo + 31u) / 32u;
    // the previous gene's p-values (first slab only): kPvWarps warps, then they join the chunks
    if (pv_tk && (threadIdx.x >> 5) < (unsigned)kPvWarps) pvalue_tiles(pv_tk, pv_c, s_pvq, erfc_table);
    auto resolve_listed = [&](uint32_t b) {
        const uint32_t sb = (b == blo) ? base : hall[b - 1];
        const uint32_t m = hall[b] - sb;
        if (m <= 65535u) resolve_big<K, false, SH, SH && !RM>(sb - base, m, href[b], ek, eg, acc, cnt, tref);
        else resolve_big<K, true, SH, false>(sb - base, m, href[b], ek, eg, acc, wide_cnt, tref);
    };
    for (;;) {
        uint32_t ch = 0;
        if (lane == 0) ch = atomicAdd(s_chunk, 1u);
        ch = __shfl_sync(0xffffffffu, ch, 0);
        if (ch >= nchunks) break;
        const uint32_t b = blo + 32u * ch + lane;
        uint32_t sb = 0, m = 0, rb = 0;
        if (b < bhi) {
            sb = (b == blo) ? base : hall[b - 1];
            m = hall[b] - sb;
            rb = href[b];
        }
        const uint32_t s0 = sb - base;
        if (m == 1u) {
            const uint32_t g = eg[s0];
            if (g) acc_add<SH>(&acc.A[g], 2ull * rb);  // a lone target value: no reference tie
        }
        bool spill = false;
        if (m > (uint32_t)kMediumBucket) {
            const uint32_t slot = atomicAdd(s_nbig, 1u);
            if (slot < biglist_cap) biglist[slot] = b;
            else spill = true;  // list full (the sizing rules this out): resolve below
        }
        // buckets of 2..32 elements, packed whole into rounds: a round takes the next
        // buckets (in order) whose sizes sum to at most 32; lane j holds the round's j-th
        // element, and the round's bucket boundaries come from the buckets' exclusive
        // prefix P over the packable sizes
        const bool pk = m >= 2u && m <= (uint32_t)kMediumBucket;
        unsigned rem = __ballot_sync(0xffffffffu, pk);
        if (rem) {
            const uint32_t mp = pk ? m : 0u;
            const uint32_t P = warp_incl_scan(mp) - mp;
            __syncwarp();  // the previous chunk's rounds have read the table
            if (pk) tbl[__popc(rem & ((1u << lane) - 1u))] = (uint8_t)lane;
            __syncwarp();
            uint32_t ord0 = 0;  // packable buckets of this chunk resolved in earlier rounds
            while (rem) {
                const int f = __ffs((int)rem) - 1;
                const uint32_t B0 = __shfl_sync(0xffffffffu, P, f);
                const bool inr = ((rem >> lane) & 1u) && P + m - B0 <= 32u;
                const unsigned I = __ballot_sync(0xffffffffu, inr);
                const unsigned starts = __reduce_or_sync(0xffffffffu, inr ? (1u << (P - B0)) : 0u);
                const int last = 31 - __clz((int)I);
                const uint32_t total = __shfl_sync(0xffffffffu, P + m, last) - B0;
                const bool active = (uint32_t)lane < total;
                int src = lane;
                if (active) src = tbl[ord0 + __popc(starts & ((2u << lane) - 1u)) - 1u];
                const uint32_t sq = __shfl_sync(0xffffffffu, s0, src);
                const uint32_t rq = __shfl_sync(0xffffffffu, rb, src);
                const uint32_t pq = __shfl_sync(0xffffffffu, P, src) - B0;
                const uint32_t mq = __shfl_sync(0xffffffffu, m, src);
                K key = K(0);
                uint32_t g = 0;
                if (active) {
                    const uint32_t e = (uint32_t)lane - pq;
                    key = ek[sq + e];
                    g = eg[sq + e];
                }
                const unsigned sub = (mq >= 32u ? 0xffffffffu : ((1u << mq) - 1u)) << pq;
                resolve_round<K, SH, RM>(active, key, g, sub, rq, acc, cnt, tref);
                ord0 += __popc(I);
                rem &= ~I;
            }
        }
        unsigned over = __ballot_sync(0xffffffffu, spill);
        while (over) {
            const int j = __ffs((int)over) - 1;
            over &= over - 1u;
            const uint32_t mj = __shfl_sync(0xffffffffu, m, j);
            const uint32_t sj = __shfl_sync(0xffffffffu, s0, j);
            const uint32_t rj = __shfl_sync(0xffffffffu, rb, j);
            if (mj <= 65535u) resolve_big<K, false, SH, SH && !RM>(sj, mj, rj, ek, eg, acc, cnt, tref);
            else resolve_big<K, true, SH, false>(sj, mj, rj, ek, eg, acc, wide_cnt, tref);
        }
    }
    // Big buckets: a warp whose chunks are done takes listed buckets while other warps may
    // still be listing (no barrier between the phases). An entry is published by its slot
    // (s_nbig) and then its bucket id; a taker that finds the id marks the entry taken. A taker
    // that finds it not yet published goes to the barrier (by default: on the screen and exact
    // workloads that is 1% and 7% faster than waiting) or, with `wait_polls`, polls for it a
    // bounded number of times. When every warp has finished its chunks and the taker's index is
    // past the final count, the list is exhausted. The pass after the barrier resolves every
    // entry not marked taken.
    __threadfence_block();
    __syncwarp();
    if (lane == 0) atomicAdd(s_wdone, 1u);
    const uint32_t nwarps = blockDim.x >> 5;
    const uint32_t pv_ntiles = pv_tk ? ((uint32_t)pv_tk->G + 30u) / 32u : 0u;
    for (;;) {
        if (pv_tk) {  // no listed bucket to take yet while chunks still run: a p-value tile instead
            uint32_t q = 0xffffffffu;
            if (lane == 0 && *(volatile uint32_t*)s_bigi >= min(*(volatile uint32_t*)s_nbig, biglist_cap) &&
                *(volatile uint32_t*)s_wdone < nwarps && *(volatile uint32_t*)s_pvq < pv_ntiles)
                q = atomicAdd(s_pvq, 1u);
            q = __shfl_sync(0xffffffffu, q, 0);
            if (q < pv_ntiles) {
                pvalue_tile(pv_tk, pv_c, q, erfc_table);
                continue;
            }
        }
        uint32_t b = kInvalid, st = 0;  // st: 0 a bucket, 1 list exhausted, 2 wait ran out
        if (lane == 0) {
            const uint32_t q = atomicAdd(s_bigi, 1u);
            for (int it = 0;; ++it) {
                const uint32_t nb = min(*(volatile uint32_t*)s_nbig, biglist_cap);
                if (q < nb) {
                    const uint32_t v = ((volatile uint32_t*)biglist)[q];
                    if (v != kInvalid) {
                        b = v;
                        biglist[q] = kTaken;
                        break;
                    }
                } else if (*(volatile uint32_t*)s_wdone == nwarps) {
                    __threadfence_block();
                    if (q >= min(*(volatile uint32_t*)s_nbig, biglist_cap)) { st = 1; break; }
                    continue;
                }
                if (it >= wait_polls) { st = 2; break; }
                __nanosleep(64);
            }
        }
        st = __shfl_sync(0xffffffffu, st, 0);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (st != 0u) break;
        resolve_listed(b);
    }
    __syncthreads();
    const uint32_t nbig = min(*s_nbig, biglist_cap);
    for (uint32_t q = threadIdx.x >> 5; q < nbig; q += nwarps) {
        const uint32_t v = biglist[q];
        if (v != kTaken && v != kInvalid) resolve_listed(v);
    }
    __syncthreads();
    // ready for the next slab (whose scatter barrier orders these before its rank phase)
    for (uint32_t q = threadIdx.x; q < nbig; q += blockDim.x) biglist[q] = kInvalid;
    if (threadIdx.x == 0) { *s_chunk = 0u; *s_nbig = 0u; *s_bigi = 0u; *s_wdone = 0u; }
}

// ---------------------------------------------------------------------------------------
// Bucket function of a gene. Buckets only need to be non-decreasing in the value (keys inside
// a bucket are compared exactly), so the kernel picks, per gene:
//   - (key - kmin) >> shift over the order keys. For floats the key bits are logarithmic in the
//     value, which suits positive data (counts, log-expression) at any scale;
//   - for a gene whose float values take both signs, (m(x) - m(xmin)) >> shift with
//         m(x) = 2^(W-1) +- u(|x|),  u(t) = floor(t * 2^(M - E0))           for t <  2^E0
//                                     u(t) = bits(t) - bits(2^E0) + 2^M    for t >= 2^E0
//     (M mantissa bits, W key bits, 2^E0 = 2^-12 of min(|xmin|, |xmax|)): linear around zero,
//     logarithmic beyond. Key bits alone would spend most buckets on the many binades of tiny
//     magnitudes, leaving values near +-1 in a few large buckets of many distinct keys.
// ---------------------------------------------------------------------------------------
template <class V>
struct BucketMap {
    using K = typename Val<V>::Key;
    static constexpr bool kFloat = std::is_same_v<V, float> || std::is_same_v<V, double>;
    static constexpr int kKeyMap = -100000;  // e0 of the plain key map
    K base = 0;                // kmin, or m(xmin)
    int shift = 0;
    int e0 = kKeyMap;          // E0 of the signed map (kKeyMap: the key map)
    __device__ __forceinline__ bool vmap() const { return e0 != kKeyMap; }
    __device__ __forceinline__ K m_of(K key) const {
        if constexpr (std::is_same_v<V, float>) {
            const float x = f32_of_key(key), t = fabsf(x);
            const uint32_t bits = __float_as_uint(t), b0 = (uint32_t)(e0 + 127) << 23;
            const uint32_t u = bits >= b0 ? bits - b0 + (1u << 23)
                                          : (uint32_t)(t * __uint_as_float((uint32_t)(23 - e0 + 127) << 23));
            return x < 0.0f ? 0x80000000u - u : 0x80000000u + u;
        } else if constexpr (std::is_same_v<V, double>) {
            const double x = f64_of_key(key), t = fabs(x);
            const unsigned long long bits = (unsigned long long)__double_as_longlong(t);
            const unsigned long long b0 = (unsigned long long)(e0 + 1023) << 52;
            const unsigned long long u = bits >= b0 ? bits - b0 + (1ull << 52)
                : (unsigned long long)(t * __longlong_as_double((long long)(52 - e0 + 1023) << 52));
            return x < 0.0 ? 0x8000000000000000ull - u : 0x8000000000000000ull + u;
        } else {
            return key;
        }
    }
    // VM: the signed map (the caller picks it once per gene, outside its loops)
    template <bool VM>
    __device__ __forceinline__ uint32_t at(K key) const {
        if constexpr (VM && kFloat) return (uint32_t)((m_of(key) - base) >> shift);
        else return (uint32_t)((key - base) >> shift);
    }
    // whether a gene with key range [kmin, kmax] takes the signed map
    static __device__ __forceinline__ bool signed_range(K kmin, K kmax) {
        if constexpr (kFloat) {
            const K k0 = Val<V>::key(V(0));
            return kmin < k0 && kmax > k0;
        } else {
            return false;
        }
    }
    // the bucket function of a gene with key range [kmin, kmax] and 2^nbl buckets
    __device__ __forceinline__ void setup(K kmin, K kmax, int nbl) {
        e0 = kKeyMap;
        base = kmin;
        K hi = kmax;
        if constexpr (kFloat) {
            if (signed_range(kmin, kmax)) {
                // the smaller of the two extreme magnitudes: an outlier on one side does not
                // stretch the linear part over the bulk of the values
                const double amag = fmin(fabs(Val<V>::from_key(kmin)), fabs(Val<V>::from_key(kmax)));
                const int ea = (int)(((unsigned long long)__double_as_longlong(amag) >> 52) & 0x7ff) - 1022;
                // 2^E0 = 2^-12 of that magnitude, kept where 2^(M - E0) is a normal number
                e0 = std::is_same_v<V, float> ? max(ea - 12, -100) : max(ea - 12, -960);
                base = m_of(kmin);
                hi = m_of(kmax);
            }
        }
        shift = 0;
        if (base <= hi) {
            const int bl = bit_length(K(hi - base));
            shift = bl > nbl ? bl - nbl : 0;
        }
    }
};

// ---------------------------------------------------------------------------------------
// Histogram path, for genes whose stored values are small integers (UMI counts): one shared-
// memory counter per (integer value, group), filled by one atomic per stored element in a
// single streaming pass over the column (no decoded copy, no bucket scatter), then
//     R[v]  = reference elements below value v    (exclusive block scan of row 0)
//     r_v   = reference elements equal to v
//     A[g]  = sum_v s_vg (2 R[v] + r_v),  B[g] = sum_v tie_delta(r_v, s_vg),  T_ref = sum_v r_v^3 - r_v
// with s_vg the count of group g at v: the same integers the bucket path accumulates (the
// reference's merge, mannwhitneyu.cpp:728-788), read off the counts, so the finalize is shared.
// The counters of row g start at word 4 + g * Vp (row 0 at 0, with room for the scan's total).
// A gene takes this path when its values are small integers (column flag), its value span V
// is at most kHistMaxBins, and the V x G counters fit in the bucket-table + element region
// and are not far more than its entries (hist_choice).
// ---------------------------------------------------------------------------------------
constexpr int kHistMaxBins = 8191;  // the block scan holds 8 entries per thread, V + 1 <= 8192

__device__ __forceinline__ long long hist_words(int Vp, int G) {
    return 4ll + (long long)G * Vp;
}
// Chooses the histogram path: span V of the integer values, the counters' words against the
// region and against the gene's entries (each counter costs about a third of an entry).
__device__ __forceinline__ bool hist_choice(long long lo, long long hi, int G, uint32_t nraw,
                                            long long region_words, int* V, int* Vp) {
    const long long span = hi - lo + 1;
    if (span < 1 || span > kHistMaxBins) return false;
    const int vp = (int)((span + 3) & ~3ll);
    const long long w = hist_words(vp, G);
    if (w > region_words || w > 3ll * nraw + 8192) return false;
    *V = (int)span;
    *Vp = vp;
    return true;
}

// Exclusive prefix sum of x[0..L) in place, x[L] = total (L < 8 * NT; x 16-byte aligned).
template <int NT>
__device__ void block_scan1(uint32_t* x, int L, uint32_t* ws) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int beg = min(L, tid * 8), cnt = min(L, beg + 8) - beg;
    uint32_t v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = i < cnt ? x[beg + i] : 0u;
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) sum += v[i];
    const uint32_t inc = warp_incl_scan(sum);
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    const uint32_t u = lane < NT / 32 ? ws[lane] : 0u;
    const uint32_t pu = warp_incl_scan(u);
    uint32_t o = __shfl_sync(0xffffffffu, pu - u, warp) + inc - sum;
    if (warp == 0 && lane == 31) x[L] = pu;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        if (i < cnt) x[beg + i] = o;
        o += v[i];
    }
    __syncthreads();
}

// Bin of a small-integer value (|v| < 2^31, as the column flag guarantees) relative to the
// gene's smallest value: converted in the value's own type, so that float data does not go
// through double (conversions to and from double take the narrow FP64 pipe).
template <class V>
__device__ __forceinline__ uint32_t hist_bin(V v, long long lo) {
    if constexpr (std::is_same_v<V, float>) return (uint32_t)(__float2int_rz(v) - (int32_t)lo);
    else if constexpr (std::is_same_v<V, double>) return (uint32_t)(__double2int_rz(v) - (int32_t)lo);
    else return (uint32_t)((long long)v - lo);
}

// One gene on the histogram path (hc: the counter region, 16-byte aligned); returns this
// thread's share of T_ref. Not inlined, so that its registers stay out of the bucket path's
// allocation. The caller's next block barrier orders its reads of the counters before the
// region is cleared for the next gene.
template <class V, int NT, class GT>
static __device__ __noinline__ unsigned long long hist_gene(
        uint32_t* hc, int hV, int hVp, long long hv0, int G, int zh, uint32_t nraw,
        const int32_t* rows, const V* data, const GT* gidp, uint32_t nrows, Acc acc,
        uint32_t* nz, uint32_t* ng, uint32_t* ws, const RankTask* pv_tk, int pv_c,
        uint32_t* s_pvq, const double* erfc_table) {
    constexpr uint32_t kNoGroup = (uint32_t)(GT)~GT(0);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int words = (int)hist_words(hVp, G);
    for (int i = 4 * tid; i < words; i += 4 * NT)
        *reinterpret_cast<uint4*>(hc + i) = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    // the previous gene's p-values: one warp per pending tile (at most kPvWarps) takes them
    // while the other warps count, as on the bucket path (a barrier between the two would make
    // every warp wait for the tiles' FP64 chains)
    const int pvw = pv_tk ? min(kPvWarps, (pv_tk->G + 30) / 32) : 0;
    if (warp < pvw) {
        pvalue_tiles(pv_tk, pv_c, s_pvq, erfc_table);
    } else {
    // one streaming pass: each stored element increments its (value, group) counter; the row
    // ids and values of the next four elements are in flight while the current ones' group ids
    // are gathered and counted (the counting threads are those of warps pvw..)
    const uint32_t nthr = (uint32_t)(NT - 32 * pvw), t0 = (uint32_t)(tid - 32 * pvw);
    int32_t r[4];
    V v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t e = t0 + (uint32_t)k * nthr;
        r[k] = e < nraw ? __ldcs(rows + e) : -1;
        v[k] = e < nraw ? ld_stream(data + e) : V(0);
    }
    for (uint32_t i = t0; i < nraw; i += 4u * nthr) {
        int32_t rn[4];
        V vn[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t e = i + 4u * nthr + (uint32_t)k * nthr;
            rn[k] = e < nraw ? __ldcs(rows + e) : -1;
            vn[k] = e < nraw ? ld_stream(data + e) : V(0);
        }
        uint32_t gl[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            gl[k] = (uint32_t)r[k] < nrows ? (uint32_t)__ldg(gidp + r[k]) : kNoGroup;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool ok = gl[k] != kNoGroup && Val<V>::finite(v[k]) &&
                            (zh == ZH_NONE || !Val<V>::zero(v[k]));
            if (ok) {
                const uint32_t bin = hist_bin<V>(v[k], hv0);
                red_add<true>(&hc[(gl[k] ? 4u + gl[k] * (uint32_t)hVp : 0u) + bin], 1u);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) { r[k] = rn[k]; v[k] = vn[k]; }
    }
    }  // counting warps
    __syncthreads();
    block_scan1<NT>(hc, hV, ws);  // hc[v] = reference elements below v, hc[V] = all of them
    // one warp per target group: its row against the reference's prefix counts
    for (int g = 1 + warp; g < G; g += NT / 32) {
        const uint32_t* row = hc + 4 + (size_t)g * hVp;
        unsigned long long sa = 0, sb = 0;
        uint32_t snz = 0, sng = 0;
        for (int v = lane; v < hV; v += 32) {
            const uint32_t sv = row[v];
            if (sv) {
                const uint32_t R = hc[v], rv = hc[v + 1] - R;
                sa += (unsigned long long)sv * (2ull * R + rv);
                sb += tie_delta(rv, sv);
                snz += sv;
                if (hv0 + v < 0) sng += sv;
            }
        }
        sa = warp_sum_u64(sa);
        sb = warp_sum_u64(sb);
        snz = __reduce_add_sync(0xffffffffu, snz);
        sng = __reduce_add_sync(0xffffffffu, sng);
        if (lane == 0) { acc.A[g] = sa; acc.B[g] = sb; nz[g] = snz; ng[g] = sng; }
    }
    unsigned long long tref = 0ull;
    for (int v = tid; v < hV; v += NT) {
        const unsigned long long rv = hc[v + 1] - hc[v];
        tref += rv * rv * rv - rv;
    }
    if (tid == 0) {
        nz[0] = hc[hV];
        ng[0] = hv0 < 0 ? hc[(int)min(-hv0, (long long)hV)] : 0u;
    }
    return tref;
}

// Finalize of one gene (threads take targets 1 + tid, 1 + tid + NT, ...): the zero block,
// U1 and the (masked) tie sum per target from the accumulators A (doubled U2 terms of the
// stored elements), B (target tie terms), the stored counts nz and negatives ng, and T_ref;
// zero_handling none also writes the per-test sample sizes. Sample-size errors and duplicate
// row ids go to the task's error words (lowest gene * G + group wins).
template <int NT>
__device__ __forceinline__ void finalize_gene(const RankTask* tk, int c, int G, int zh, const Acc& acc,
                                              const uint32_t* nz, const uint32_t* ng,
                                              unsigned long long T_ref) {
    const unsigned long long nz1 = nz[0];
    for (int g = 1 + (int)threadIdx.x; g < G; g += NT) {
        const size_t idx = (size_t)(g - 1) * tk->n_cols + c;
        const unsigned long long nz2 = nz[g];
        unsigned long long n1, n2, u2x2, ties;
        if (zh == ZH_NONE) {
            n1 = nz1;
            n2 = nz2;
            if (n1 < 2) atomicMin(&tk->err[0], (unsigned long long)c * G);
            else if (n2 < 2) atomicMin(&tk->err[0], (unsigned long long)c * G + g);
            u2x2 = acc.A[g];
            ties = T_ref + acc.B[g];
            tk->n2[idx] = (uint32_t)nz2;
            if (g == 1) tk->n1[c] = (uint32_t)nz1;
        } else {
            n1 = (unsigned long long)tk->group_rows[0];
            n2 = (unsigned long long)tk->group_rows[g];
            if (nz1 > n1) atomicMin(&tk->err[1], (unsigned long long)c * G);
            if (nz2 > n2) atomicMin(&tk->err[1], (unsigned long long)c * G + g);
            const unsigned long long z1 = n1 - nz1, z2 = n2 - nz2;
            if (zh == ZH_MIN) u2x2 = acc.A[g] + 2ull * z1 * nz2 + z1 * z2;
            else if (zh == ZH_MAX) u2x2 = acc.A[g] + z2 * (2ull * nz1 + z1);
            else u2x2 = acc.A[g] + 2ull * z1 * (nz2 - ng[g]) + z2 * (2ull * ng[0] + z1);
            const unsigned long long zz = z1 + z2;
            ties = T_ref + acc.B[g] + zz * zz * zz - zz;
        }
        const long long u1x2 = (long long)(2ull * n1 * n2) - (long long)u2x2;
        tk->U1[idx] = (double)u1x2 * 0.5;
        tk->tie[idx] = tk->tie_correction ? (double)ties : 0.0;
    }
}

// HIST: the variant with the histogram path (launched when some column of the launch's tasks
// can hold small integers; without it the bucket path keeps its register allocation).
// CPX: the variant that can compact its decoded copy (launched when a task of the launch asks
// for it, RankTask::compact_decode).
// RM: accumulators in shared memory, run counters in global memory (large G: the shared memory
// goes to elements; rounds resolve repeated groups by warp match).
template <class V, int NT, bool ACC_SMEM, bool HIST, bool CPX, bool RM>
__global__ void __launch_bounds__(NT, 1) mwu_rank_kernel(const RankArgs a) {
    using K = typename Val<V>::Key;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_gene, s_task;
    __shared__ unsigned long long s_tref;
    __shared__ uint32_t s_maxb, s_slab_hi, s_chunk, s_nbig, s_bigi, s_wdone;
    __shared__ uint32_t s_ndec;  // entries of the compacted decoded copy
    __shared__ int s_pv_gene, s_pv_task;  // gene whose p-values are pending (-1: none)
    __shared__ uint32_t s_pvq;            // its p-value tiles taken so far
    // the next gene and its column metadata, fetched during the current gene's finalize by a
    // thread that has no target to finalize, so that the work-queue atomic and the dependent
    // loads are off the critical path
    __shared__ int s_next_gene, s_next_task;
    __shared__ long long s_next_p0, s_next_p1;
    __shared__ unsigned long long s_next_kmin, s_next_kmax;
    __shared__ uint32_t s_next_hz;
    __shared__ uint32_t s_wsx[32], s_wsy[32];
    __shared__ uint8_t s_tbl[NT / 32][32];  // per warp: packable bucket -> lane (rank rounds)

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wait_polls = a.drain_wait ? kDrainWaitIters : 0;
    const int GL = a.G;  // layout G
    const int NBMAX = 1 << a.nb_max_log2;
    constexpr bool CNT_SMEM = ACC_SMEM && !RM;
    const RankSmem L(a.nb_max_log2, GL, a.tie_warps, ACC_SMEM, CNT_SMEM, a.elem_smem_cap,
                     (int)sizeof(K));
    const int cw = RankSmem::cnt_words(GL);

    uint32_t* hall = reinterpret_cast<uint32_t*>(smem + L.acc_bytes + L.cnt_bytes);  // bucket
                                                         // start (after the scan)
    uint32_t* href = hall + NBMAX + 4;                   // reference elements below a bucket
    uint32_t* biglist = href + NBMAX + 4;                // large buckets of the current slab
    const uint32_t biglist_cap = (uint32_t)RankSmem::big_list(
        RankSmem::compact_cap(a.elem_smem_cap, (int)sizeof(K), ACC_SMEM));
    unsigned char* accb;
    uint32_t* cnt_base;
    const size_t cta = (size_t)a.cta_base + blockIdx.x;  // this CTA's scratch slices
    uint32_t* cnt_glob = a.cnt_global + cta * a.tie_warps * (cw + GL);
    if constexpr (ACC_SMEM) {
        accb = smem;
        cnt_base = CNT_SMEM ? reinterpret_cast<uint32_t*>(smem + L.acc_bytes) : cnt_glob;
    } else {
        accb = a.acc_global + cta * 24 * GL;
        cnt_base = cnt_glob;
    }
    unsigned long long* A = reinterpret_cast<unsigned long long*>(accb);
    unsigned long long* B = A + GL;
    uint32_t* nz = reinterpret_cast<uint32_t*>(B + GL);
    uint32_t* ng = nz + GL;
    const Acc acc{A, B};
    uint32_t* wide_base = cnt_glob + (size_t)a.tie_warps * cw;
    uint32_t* cnt = cnt_base + (size_t)warp * cw;
    uint32_t* wide_cnt = wide_base + (size_t)warp * GL;
    using GT = GroupType<ACC_SMEM>;
    constexpr uint32_t kNoGroup = ACC_SMEM ? 0xffffu : 0xffffffffu;
    // the element region holds a slab either with full keys (cap_full elements) or, when a
    // bucket spans at most 2^16 keys, with 16-bit offsets of the key inside its bucket
    // (cap_compact elements): within a bucket the offsets order like the keys
    unsigned char* elem_base = smem + L.acc_bytes + L.cnt_bytes + L.hist_bytes;
    const uint32_t cap_full = (uint32_t)a.elem_smem_cap;
    const uint32_t cap_compact = (uint32_t)RankSmem::compact_cap(a.elem_smem_cap, (int)sizeof(K), ACC_SMEM);
    K* ek_s = reinterpret_cast<K*>(elem_base);
    GT* eg_s = reinterpret_cast<GT*>(ek_s + cap_full);
    uint16_t* eo_s = reinterpret_cast<uint16_t*>(elem_base);
    GT* ego_s = reinterpret_cast<GT*>(eo_s + cap_compact);
    K* dk = reinterpret_cast<K*>(a.dk_global) + cta * a.slice;
    GT* dg = reinterpret_cast<GT*>(a.dg_global) + cta * a.slice;
    K* ek_g = reinterpret_cast<K*>(a.ek_global) + cta * a.slice;
    GT* eg_g = reinterpret_cast<GT*>(a.eg_global) + cta * a.slice;

    for (int i = tid; i < a.tie_warps * cw; i += NT) cnt_base[i] = 0u;
    for (int i = tid; i < a.tie_warps * GL; i += NT) wide_base[i] = 0u;
    for (uint32_t i = tid; i < biglist_cap; i += NT) biglist[i] = kInvalid;
    if (tid == 0) {
        s_chunk = 0u; s_nbig = 0u; s_bigi = 0u; s_wdone = 0u;
        s_pv_gene = -1; s_pv_task = 0; s_pvq = 0u;
    }

    bool first = true;  // (thread NT - 1) the plain form's one gene is still to be handed out
    auto fetch_next = [&]() {
        int c = -1, ti = 0;
        if (a.single_gene >= 0) {
            c = first ? a.single_gene : -1;
            first = false;
        } else {
            const int gi = atomicAdd(a.queue, 1);
            if (gi < a.n_order) {
                c = a.order[gi];
                ti = a.order_task ? (int)a.order_task[gi] : 0;
            }
        }
        s_next_gene = c;
        s_next_task = ti;
        if (c >= 0) {
            const RankTask* t = a.tasks + ti;
            s_next_p0 = t->indptr[c];
            s_next_p1 = t->indptr[c + 1];
            s_next_kmin = t->col_kmin[c];
            s_next_kmax = t->col_kmax[c];
            s_next_hz = t->col_has_zero[c];
        }
    };
    if (tid == NT - 1) fetch_next();
    for (int b = tid; b <= NBMAX; b += NT) { hall[b] = 0u; href[b] = 0u; }
    __syncthreads();

    for (;;) {
        if (tid == 0) {
            s_gene = s_next_gene;
            s_task = s_next_task;
            s_tref = 0ull;
            s_maxb = 0u;
            s_ndec = 0u;
        }
        for (int g = tid; g < GL; g += NT) { A[g] = 0ull; B[g] = 0ull; nz[g] = 0u; ng[g] = 0u; }
        __syncthreads();
        const int c = s_gene;
        const int pv_c = s_pv_gene;
        const RankTask* pv_tk = (a.erfc_table && pv_c >= 0) ? a.tasks + s_pv_task : nullptr;
        if (c < 0) {
            if (pv_tk) pvalue_tiles(pv_tk, pv_c, &s_pvq, a.erfc_table);
            break;
        }
        const RankTask* tk = a.tasks + s_task;
        const int G = tk->G, zh = tk->zero_handling;
        const GT* gidp = reinterpret_cast<const GT*>(tk->group_of_row);
        const uint32_t nrows = (uint32_t)tk->n_rows;
        const long long p0 = s_next_p0;
        const uint32_t nraw = (uint32_t)(s_next_p1 - p0);
        // entries of this gene, re-based: entry i is rows[i], data[i]; its decoded copy is
        // dk/dg[i]. Passes over the entries go by warp tiles of 128: lane l of a warp takes
        // entries t + l + 32k (k < 4), so that neighbouring lanes read neighbouring entries
        // and their group-id gathers (rows of one column ascend) share L2 sectors.
        const int32_t* rows = tk->rows + p0;
        const V* data = reinterpret_cast<const V*>(tk->data) + p0;

        // ---- bucket function from the column's key range ----
        K kmin = (K)s_next_kmin, kmax = (K)s_next_kmax;
        if (zh == ZH_NONE && (s_next_hz & 1u)) {
            const K kz = Val<V>::key(V(0));
            kmin = kz < kmin ? kz : kmin;
            kmax = kz > kmax ? kz : kmax;
        }
        int nbl = 1;
        while (nbl < a.nb_max_log2 && (1u << nbl) < 2u * nraw) ++nbl;
        const int NB = 1 << nbl;
        // bucket map: the key map ((key - kmin) >> shift) or, for signed float genes, the signed
        // map, whose constants the instantiations below rebuild where they need them
        const bool vmap = BucketMap<V>::signed_range(kmin, kmax);
        int shift;
        {
            BucketMap<V> bm;
            bm.setup(kmin, kmax, nbl);
            shift = bm.shift;
        }
        // (the bucket table is all zeros here: zeroed before the first gene, and each gene
        // clears the entries it used while it finalizes)

        // ---- path: histogram (small integer values) or buckets ----
        int hV = 0, hVp = 0;
        long long hv0 = 0;
        bool use_hist = false;
        if constexpr (ACC_SMEM && HIST) {
            if (!a.no_histogram && !(s_next_hz & 2u) && kmin <= kmax) {
                hv0 = (long long)Val<V>::from_key(kmin);
                use_hist = hist_choice(hv0, (long long)Val<V>::from_key(kmax), G, nraw,
                                       (long long)((L.hist_bytes + L.elem_bytes) / 4), &hV, &hVp);
            }
        }
        unsigned long long tref = 0ull;
        if (HIST && use_hist) {
            tref = hist_gene<V, NT, GT>(hall, hV, hVp, hv0, G, zh, nraw, rows, data, gidp, nrows,
                                        acc, nz, ng, s_wsx, pv_tk, pv_c, &s_pvq, a.erfc_table);
        } else {
        // ---- pass 1 (HBM): decode to (key, group), histograms, per-group counts ----
        uint32_t nref_local = 0;
        // (instantiated for each bucket map, chosen once per gene)
        auto pass1 = [&](auto vm_tag, auto cp_tag) {
            constexpr bool VM = decltype(vm_tag)::value;
            constexpr bool CP = decltype(cp_tag)::value;  // compacted decoded copy
            BucketMap<V> bmap;
            if constexpr (VM) bmap.setup(kmin, kmax, nbl);
            else { bmap.base = kmin; bmap.shift = shift; }
            uint32_t t = 128u * (uint32_t)warp;
            if (t < nraw) {
                int32_t r[4];
                V v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t i = t + 32u * k + lane;
                    r[k] = i < nraw ? __ldcs(rows + i) : -1;
                    v[k] = i < nraw ? ld_stream(data + i) : V(0);
                }
                for (;;) {
                    const uint32_t tn = t + 4u * NT;
                    const bool more = tn < nraw;
                    int32_t rn[4];
                    V vn[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const uint32_t i = tn + 32u * k + lane;
                        rn[k] = (more && i < nraw) ? __ldcs(rows + i) : -1;
                        vn[k] = (more && i < nraw) ? ld_stream(data + i) : V(0);
                    }
                    // all four group-id gathers in flight before any of them is tested
                    uint32_t gl[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        gl[k] = (uint32_t)r[k] < nrows ? (uint32_t)__ldg(gidp + r[k]) : kNoGroup;
                    // compacted copy: the warp's stored entries of these 4 rounds take
                    // consecutive positions (one atomic per warp)
                    uint32_t cpos = 0;
                    unsigned okm[4];
                    if constexpr (CP) {
                        uint32_t tot = 0;
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            okm[k] = __ballot_sync(0xffffffffu, gl[k] != kNoGroup && Val<V>::finite(v[k]) &&
                                                                    (zh == ZH_NONE || !Val<V>::zero(v[k])));
                            tot += __popc(okm[k]);
                        }
                        if (lane == 0 && tot) cpos = atomicAdd(&s_ndec, tot);
                        cpos = __shfl_sync(0xffffffffu, cpos, 0);
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const uint32_t i = t + 32u * k + lane;
                        const bool ok = gl[k] != kNoGroup && Val<V>::finite(v[k]) &&
                                        (zh == ZH_NONE || !Val<V>::zero(v[k]));
                        const K key = ok ? Val<V>::key(v[k]) : K(0);
                        const uint32_t g = ok ? gl[k] : kNoGroup;
                        if constexpr (CP) {
                            if (ok) {
                                const uint32_t q = cpos + __popc(okm[k] & ((1u << lane) - 1u));
                                dk[q] = key;
                                dg[q] = (GT)g;
                            }
                            cpos += __popc(okm[k]);
                        } else {
                            if (i < nraw) { dk[i] = key; dg[i] = (GT)g; }
                        }
                        if (ok) {
                            if (g) red_add<ACC_SMEM>(&nz[g], 1u);
                            else ++nref_local;
                            if (zh == ZH_MIX && Val<V>::neg(v[k])) red_add<ACC_SMEM>(&ng[g], 1u);
                            const uint32_t b = bmap.template at<VM>(key);
                            red_add<true>(&hall[b], 1u);
                            if (g == 0) red_add<true>(&href[b], 1u);
                        }
                    }
                    if (!more) break;
                    t = tn;
#pragma unroll
                    for (int k = 0; k < 4; ++k) { r[k] = rn[k]; v[k] = vn[k]; }
                }
            }
        };
        const bool cdec = CPX && tk->compact_decode != 0;
        if constexpr (CPX) {
            if (vmap) {
                if (cdec) pass1(std::true_type{}, std::true_type{});
                else pass1(std::true_type{}, std::false_type{});
            } else {
                if (cdec) pass1(std::false_type{}, std::true_type{});
                else pass1(std::false_type{}, std::false_type{});
            }
        } else {
            if (vmap) pass1(std::true_type{}, std::false_type{});
            else pass1(std::false_type{}, std::false_type{});
        }
        nref_local = __reduce_add_sync(0xffffffffu, nref_local);
        if (lane == 0 && nref_local) red_add<ACC_SMEM>(&nz[0], nref_local);
        __syncthreads();
        block_scan2<NT>(hall, href, NB, s_wsx, s_wsy, &s_maxb);
        const uint32_t n = hall[NB];
        const uint32_t ndec = cdec ? s_ndec : nraw;  // entries of the decoded copy
        // 16-bit key offsets inside a bucket: the buckets of the key map hold keys that differ
        // in their low `shift` bits only
        const bool compact = !vmap && shift <= 16;
        const uint32_t cap = compact ? cap_compact : cap_full;
        const K offmask = compact ? (K)((1u << shift) - 1u) : K(0);
        // slabs: the whole gene when it fits in shared memory; else buckets whose start lies
        // in [k*W, (k+1)*W) form slab k, which holds at most W + (largest bucket) elements:
        // that fits the capacity unless one bucket is larger than half of it (such a slab is
        // placed in the global slice)
        const uint32_t maxb = s_maxb;
        uint32_t W = n, nslabs = n ? 1u : 0u;
        if (n > cap && cap >= 1024u) {
            W = max(cap > maxb ? cap - maxb : 0u, cap / 2u);
            nslabs = (n - 1u) / W + 1u;
        }

        // During a slab's scatter hall[b] counts up from the start to the end of bucket b,
        // so afterwards the start of bucket b is hall[b - 1] (or the slab base for its first
        // bucket) and buckets of later slabs still hold their starts.
        uint32_t blo = 0;
        uint32_t base = 0;  // start of the slab in the gene's bucket order (elements of earlier
                            // slabs; kept here, since hall[blo] counts up during the scatter)
        for (uint32_t slab = 0; slab < nslabs; ++slab) {
            // the slab's bucket range; the last slab ends at NB. (The scan, and the previous
            // slab's rank phase, end with a block barrier.)
            uint32_t bhi = (uint32_t)NB;
            if (slab + 1u < nslabs) {
                if (tid == 0) {  // first b >= blo whose start is >= (slab + 1) * W
                    uint32_t lo = blo, hi = (uint32_t)NB;
                    const uint32_t t1 = (slab + 1u) * W;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (hall[mid] < t1) lo = mid + 1u; else hi = mid;
                    }
                    s_slab_hi = lo;
                }
                __syncthreads();
                bhi = s_slab_hi;
            }
            const uint32_t cnt_slab = hall[bhi] - base;  // hall[bhi] is outside this slab
            const bool in_smem = cnt_slab <= cap;

            // ---- pass 2 (L2): scatter this slab's decoded elements into bucket order ----
            auto scatter = [&](auto vm_tag) {
                constexpr bool VM = decltype(vm_tag)::value;
                BucketMap<V> bmap;
                if constexpr (VM) bmap.setup(kmin, kmax, nbl);
                else { bmap.base = kmin; bmap.shift = shift; }
                const bool all = nslabs == 1u;
                uint32_t t = 128u * (uint32_t)warp;
                if (t < ndec) {
                    K k4[4];
                    uint32_t g4[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const uint32_t i = t + 32u * k + lane;
                        k4[k] = i < ndec ? dk[i] : K(0);
                        g4[k] = i < ndec ? (uint32_t)dg[i] : kNoGroup;
                    }
                    for (;;) {
                        const uint32_t tn = t + 4u * NT;
                        const bool more = tn < ndec;
                        K kn[4];
                        uint32_t gn[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            const uint32_t i = tn + 32u * k + lane;
                            kn[k] = (more && i < ndec) ? dk[i] : K(0);
                            gn[k] = (more && i < ndec) ? (uint32_t)dg[i] : kNoGroup;
                        }
                        uint32_t bb[4];
                        bool in[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            bb[k] = bmap.template at<VM>(k4[k]);
                            in[k] = g4[k] != kNoGroup && (all || (bb[k] >= blo && bb[k] < bhi));
                        }
                        uint32_t pos[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (in[k]) pos[k] = atom_add<true>(&hall[bb[k]], 1u) - base;
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            if (!in[k]) continue;
                            if (!in_smem) { ek_g[pos[k]] = k4[k]; eg_g[pos[k]] = (GT)g4[k]; }
                            else if (compact) { eo_s[pos[k]] = (uint16_t)((k4[k] - kmin) & offmask); ego_s[pos[k]] = (GT)g4[k]; }
                            else { ek_s[pos[k]] = k4[k]; eg_s[pos[k]] = (GT)g4[k]; }
                        }
                        if (!more) break;
                        t = tn;
#pragma unroll
                        for (int k = 0; k < 4; ++k) { k4[k] = kn[k]; g4[k] = gn[k]; }
                    }
                }
            };
            if (cnt_slab) {
                if (vmap) scatter(std::true_type{});
                else scatter(std::false_type{});
            }
            __syncthreads();
            if (slab + 1u == nslabs) {
                // the decoded copy is dead: drop its lines from L2 instead of writing them back
                l2_discard<NT>(dk, (size_t)ndec * sizeof(K));
                l2_discard<NT>(dg, (size_t)ndec * sizeof(GT));
            }

            // ---- rank ----
            if (in_smem && compact)
                rank_slab<uint32_t, ACC_SMEM, RM>(eo_s, ego_s, blo, bhi, base, hall, href, biglist,
                                              biglist_cap, &s_chunk, &s_nbig, &s_bigi, &s_wdone, acc, cnt,
                                              wide_cnt, s_tbl[warp], tref, slab ? nullptr : pv_tk, pv_c,
                                              &s_pvq, a.erfc_table, wait_polls);
            else if (in_smem)
                rank_slab<K, ACC_SMEM, RM>(ek_s, eg_s, blo, bhi, base, hall, href, biglist,
                                       biglist_cap, &s_chunk, &s_nbig, &s_bigi, &s_wdone, acc, cnt,
                                       wide_cnt, s_tbl[warp], tref, slab ? nullptr : pv_tk, pv_c,
                                       &s_pvq, a.erfc_table, wait_polls);
            else
                rank_slab<K, ACC_SMEM, RM>(ek_g, eg_g, blo, bhi, base, hall, href, biglist,
                                       biglist_cap, &s_chunk, &s_nbig, &s_bigi, &s_wdone, acc, cnt,
                                       wide_cnt, s_tbl[warp], tref, slab ? nullptr : pv_tk, pv_c,
                                       &s_pvq, a.erfc_table, wait_polls);
            blo = bhi;
            base += cnt_slab;
        }
        }  // bucket path
        // pending p-values not taken in the rank phase (a gene without stored elements has none)
        if (pv_tk) pvalue_tiles(pv_tk, pv_c, &s_pvq, a.erfc_table);
        tref = warp_sum_u64(tref);
        if (lane == 0 && tref) atomicAdd(&s_tref, tref);
        __syncthreads();

        // ---- finalize per target ----
        // the s_next_* values of this gene were read after the barriers above; the next gene
        // is fetched now (thread NT - 1 finalizes a target only when G > NT)
        if (tid == NT - 1) fetch_next();
        finalize_gene<NT>(tk, c, G, zh, acc, nz, ng, s_tref);
        // for the next gene: a clear bucket table (all of it, and the big list, after the
        // histogram path used the region for its counters)
        const int nb_used = use_hist ? NBMAX : NB;
        for (int b = tid; b <= nb_used; b += NT) { hall[b] = 0u; href[b] = 0u; }
        if (use_hist)
            for (uint32_t q = tid; q < biglist_cap; q += NT) biglist[q] = kInvalid;
        if (tid == 0 && a.erfc_table) {  // this gene's p-values: pending until the next gene
            s_pv_gene = c;
            s_pv_task = s_task;
            s_pvq = 0u;
        }
        __syncthreads();
    }
}

// Group of every row in the rank kernel's group type: the caller's id when it names a group
// in [0, G), else all ones (the reference skips such rows, mannwhitneyu.cpp:914-926).
template <class GT>
__global__ void prepare_group_ids_kernel(const int32_t* gid, long long n_rows, int32_t G, GT* out) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += stride) {
        const int32_t g = gid[r];
        out[r] = (g >= 0 && g < G) ? (GT)g : (GT)~GT(0);
    }
}

// Per-column key range of finite nonzero values, whether an explicit finite zero is stored
// (bit 0 of has_zero) and whether a finite nonzero value is not a small integer (bit 1: the
// column cannot take the histogram path), for columns [0, n_cols) of `indptr` (entry
// positions into `data`). Entry-parallel:
// a warp takes runs of 32 * kRangePer consecutive entries, lane l the kRangePer entries from
// l * kRangePer; a lane folds the entries of one column at a time and publishes a column with
// 64-bit atomics when it leaves it (a warp whose lanes all end in one column combines them
// first). kmin / kmax / has_zero must hold all ones / 0 / 0 on entry.
constexpr int kRangePer = 16;
template <class V>
__global__ void column_key_range_kernel(const V* data, const int64_t* indptr, int32_t n_cols,
                                        unsigned long long* kmin, unsigned long long* kmax,
                                        uint32_t* has_zero) {
    using K = typename Val<V>::Key;
    if (n_cols <= 0) return;
    const long long eb = indptr[0], ee = indptr[n_cols];
    const long long span = 32ll * kRangePer;
    const long long runs = (ee - eb + span - 1) / span;
    const int lane = threadIdx.x & 31;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < runs; r += nw) {
        const long long s0 = eb + r * span + (long long)lane * kRangePer;
        const long long s1 = s0 + kRangePer < ee ? s0 + kRangePer : ee;
        int col = -1;
        K lo = ~K(0), hi = K(0);
        bool z = false, nonint = false;
        auto publish = [&](int c) {
            if (lo <= hi) {
                atomicMin(&kmin[c], (unsigned long long)lo);
                atomicMax(&kmax[c], (unsigned long long)hi);
            }
            if (z || nonint) atomicOr(&has_zero[c], (z ? 1u : 0u) | (nonint ? 2u : 0u));
            lo = ~K(0); hi = K(0); z = false; nonint = false;
        };
        if (s0 < ee) {
            int a = 0, b = n_cols - 1;  // the column holding s0: last c with indptr[c] <= s0
            while (a < b) {
                const int mid = (a + b + 1) >> 1;
                if (indptr[mid] <= s0) a = mid; else b = mid - 1;
            }
            col = a;
            long long cend = indptr[col + 1];
            for (long long e = s0; e < s1; ++e) {
                while (e >= cend) { publish(col); ++col; cend = indptr[col + 1]; }
                const V v = data[e];
                if (!Val<V>::finite(v)) continue;
                if (Val<V>::zero(v)) { z = true; continue; }
                nonint |= !Val<V>::small_int(v);
                const K k = Val<V>::key(v);
                lo = k < lo ? k : lo;
                hi = k > hi ? k : hi;
            }
        }
        const int c0 = __shfl_sync(0xffffffffu, col, 0);
        if (__all_sync(0xffffffffu, col == c0 || col < 0)) {
            lo = warp_min(lo);
            hi = warp_max(hi);
            z = __any_sync(0xffffffffu, z);
            nonint = __any_sync(0xffffffffu, nonint);
            if (lane == 0 && c0 >= 0) publish(c0);
        } else if (col >= 0) {
            publish(col);
        }
    }
}

}  // namespace hpdex
