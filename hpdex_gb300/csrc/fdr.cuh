// fdr.cuh -- the DE driver's post-processing on the device (sm_103a): Benjamini-Hochberg
// adjusted p-values over all (gene, target) tests, and fold changes from group means.
//
// BH follows scipy.stats.false_discovery_control(ps, method="bh"), which the reference DE
// driver calls (AI4Cell/hpdex src/hpdex/de.py:174-184): sort the p-values ascending, multiply
// the i-th (1-based) by m / i (one division, one multiplication, both rounded to nearest),
// replace each by the minimum of itself and everything after it, restore the input order,
// clip to [0, 1]. Equal p-values end with equal adjusted values whatever their order among
// themselves (the suffix minimum spans their whole run), so the sort need not match numpy's.
//
// The sort is a stable LSD radix sort of the p-values' bit patterns (non-negative doubles
// order like their bits) with 32-bit indices: 8 passes of 8-bit digits, each one count
// kernel (per-block digit histograms), one scan kernel (digit-major exclusive prefix over all
// blocks), one scatter kernel (per-warp stable ranks from warp match, per-warp bases from the
// block's counts).
#pragma once
#include <cstdint>

#include "common.cuh"

namespace hpdex {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;                             // per thread and tile
constexpr int kSortTile = kSortThreads * kSortItems;      // 2048 entries per block
constexpr int kSortWarps = kSortThreads / 32;

// -0.0 would sort after every positive value by its bits: make it +0.0 (they compare equal).
__global__ void canonical_zero_kernel(unsigned long long* keys, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        if (keys[i] == 0x8000000000000000ull) keys[i] = 0ull;
}

__global__ void __launch_bounds__(kSortThreads) radix_count_kernel(const unsigned long long* keys,
                                                                   long long n, int shift,
                                                                   uint32_t* counts, int nblocks) {
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0u;
    __syncthreads();
    const long long t0 = (long long)blockIdx.x * kSortTile;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const long long i = t0 + (long long)k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&hist[(uint32_t)(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
}

// In-place exclusive prefix sum of counts[0..len) (one block of 1024 threads).
__global__ void __launch_bounds__(1024) radix_scan_kernel(uint32_t* counts, long long len) {
    __shared__ uint32_t ws[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long per = (len + 1023) / 1024;
    const long long beg = min(len, (long long)tid * per), end = min(len, beg + per);
    uint32_t s = 0;
    for (long long i = beg; i < end; ++i) s += counts[i];
    const uint32_t incl = warp_incl_scan(s);
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t v = ws[lane];
        ws[lane] = warp_incl_scan(v) - v;
    }
    __syncthreads();
    uint32_t o = ws[warp] + incl - s;
    for (long long i = beg; i < end; ++i) {
        const uint32_t c = counts[i];
        counts[i] = o;
        o += c;
    }
}

// Stable scatter of one pass. vin == nullptr: the values are the input positions.
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const unsigned long long* kin, const uint32_t* vin, unsigned long long* kout, uint32_t* vout,
    long long n, int shift, const uint32_t* offsets, int nblocks) {
    __shared__ uint32_t whist[kSortWarps][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < kSortWarps * 256; d += kSortThreads) (&whist[0][0])[d] = 0u;
    __syncthreads();
    // warp w takes the tile's entries [w*256, (w+1)*256), 32 consecutive ones per round
    const long long base = (long long)blockIdx.x * kSortTile + (long long)warp * 32 * kSortItems;
    unsigned long long key[kSortItems];
    uint32_t val[kSortItems], dig[kSortItems], rank[kSortItems];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const long long i = base + r * 32 + lane;
        const bool ok = i < n;
        key[r] = ok ? kin[i] : 0ull;
        val[r] = ok ? (vin ? vin[i] : (uint32_t)i) : 0u;
        dig[r] = ok ? ((uint32_t)(key[r] >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, dig[r]);
        const uint32_t before = ok ? whist[warp][dig[r]] : 0u;
        rank[r] = before + __popc(peers & lt);
        __syncwarp();
        if (ok && (peers & lt) == 0u) whist[warp][dig[r]] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {   // per digit: bases of the warps in tile order, from the block's global offset
        const int d = threadIdx.x;
        uint32_t run = offsets[(size_t)d * nblocks + blockIdx.x];
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t c = whist[w][d];
            whist[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        if (dig[r] < 256u) {
            const uint32_t pos = whist[warp][dig[r]] + rank[r];
            kout[pos] = key[r];
            vout[pos] = val[r];
        }
    }
}

// BH, step 1: per block of sorted p-values, the minimum of the adjusted values p_(i) * (m / i).
__device__ __forceinline__ double bh_adjusted(const unsigned long long* sk, long long i, long long m) {
    const double p = __longlong_as_double((long long)sk[i]);
    return __dmul_rn(p, __ddiv_rn((double)m, (double)(i + 1)));
}

__global__ void __launch_bounds__(kSortThreads) bh_block_min_kernel(const unsigned long long* sk,
                                                                     long long m, double* agg,
                                                                     uint32_t* bad) {
    __shared__ double ws[kSortWarps];
    const long long t0 = (long long)blockIdx.x * kSortTile;
    double v = __longlong_as_double(0x7ff0000000000000ll);  // +inf
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const long long i = t0 + (long long)k * kSortThreads + threadIdx.x;
        if (i < m) {
            const double p = __longlong_as_double((long long)sk[i]);
            if (!(p >= 0.0 && p <= 1.0)) atomicOr(bad, 1u);  // NaN, negative or above 1
            v = fmin(v, bh_adjusted(sk, i, m));
        }
    }
    for (int o = 16; o; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = ws[0];
        for (int w = 1; w < kSortWarps; ++w) a = fmin(a, ws[w]);
        agg[blockIdx.x] = a;
    }
}

// BH, step 2 (one block): carry[b] = min(agg[b+1..]) (+inf for the last block).
__global__ void __launch_bounds__(1024) bh_carry_kernel(const double* agg, int nblocks, double* carry) {
    __shared__ double ws[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (nblocks + 1023) / 1024;
    // thread t owns blocks [t*per, (t+1)*per), scanned from the end
    const int beg = min(nblocks, tid * per), end = min(nblocks, beg + per);
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    double s = inf;
    for (int b = beg; b < end; ++b) s = fmin(s, agg[b]);
    // suffix min over threads: thread t needs min over threads > t
    double incl = s;  // reverse inclusive scan within the warp
    for (int o = 1; o < 32; o <<= 1) {
        const double x = __shfl_down_sync(0xffffffffu, incl, o);
        if (lane + o < 32) incl = fmin(incl, x);
    }
    if (lane == 0) ws[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        double v = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const double x = __shfl_down_sync(0xffffffffu, v, o);
            if (lane + o < 32) v = fmin(v, x);
        }
        ws[lane] = v;  // min over warps >= lane
    }
    __syncthreads();
    // min over threads after t: later lanes of this warp, then later warps
    double after = __shfl_down_sync(0xffffffffu, incl, 1);
    if (lane == 31) after = inf;
    if (warp + 1 < 32) after = fmin(after, ws[warp + 1]);
    double run = after;
    for (int b = end - 1; b >= beg; --b) {
        carry[b] = run;
        run = fmin(run, agg[b]);
    }
}

// BH, step 3: suffix minimum inside each block plus its carry, clip, back to input order.
__global__ void __launch_bounds__(kSortThreads) bh_apply_kernel(const unsigned long long* sk,
                                                                 const uint32_t* sv, long long m,
                                                                 const double* carry, double* fdr) {
    __shared__ double ws[kSortWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long t0 = (long long)blockIdx.x * kSortTile + (long long)threadIdx.x * kSortItems;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    double a[kSortItems];
    double tmin = inf;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const long long i = t0 + k;
        a[k] = i < m ? bh_adjusted(sk, i, m) : inf;
        tmin = fmin(tmin, a[k]);
    }
    // min over the threads after this one (tile order = thread order)
    double incl = tmin;
    for (int o = 1; o < 32; o <<= 1) {
        const double x = __shfl_down_sync(0xffffffffu, incl, o);
        if (lane + o < 32) incl = fmin(incl, x);
    }
    if (lane == 0) ws[warp] = incl;
    __syncthreads();
    double after = __shfl_down_sync(0xffffffffu, incl, 1);
    if (lane == 31) after = inf;
    for (int w = warp + 1; w < kSortWarps; ++w) after = fmin(after, ws[w]);
    after = fmin(after, carry[blockIdx.x]);
#pragma unroll
    for (int k = kSortItems - 1; k >= 0; --k) {
        after = fmin(after, a[k]);
        const long long i = t0 + k;
        if (i < m) fdr[sv[i]] = after < 0.0 ? 0.0 : (after > 1.0 ? 1.0 : after);
    }
}

// Fold change and log2 fold change per (target, gene) from per-(gene, group) means
// (gene-major [gene * G + g], g = 0 the reference), as the reference DE driver computes them
// (de.py:138-142): fc = tar / ref; ref < 1e-10 -> clip; then tar < 1e-10 -> 1 / clip.
__global__ void fold_change_kernel(const double* means, long long n_genes, int G, double clip,
                                   double* fold, double* log2fold) {
    const long long n = (long long)(G - 1) * n_genes;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long t = i / n_genes, c = i - t * n_genes;
        const double ref = means[c * G], tar = means[c * G + t + 1];
        double f = __ddiv_rn(tar, ref);
        if (ref < 1e-10) f = clip;
        if (tar < 1e-10) f = __ddiv_rn(1.0, clip);
        fold[i] = f;
        log2fold[i] = log2(f);
    }
}

}  // namespace hpdex
