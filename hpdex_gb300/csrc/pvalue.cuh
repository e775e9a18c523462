// pvalue.cuh -- p-value stage of the MWU backend (sm_103a).
//
// Asymptotic: mwu_pvalue_asymptotic_kernel applies the per-test arithmetic of
// pvalue_math.cuh (the reference's precise path, AI4Cell/hpdex src/cpp/mannwhitneyu.cpp:15-96,
// in the same double operation order, erfc from a table) to a column range of the rank
// kernel's outputs. The rank kernel can also run the same arithmetic itself (fused p-values).
//
// Exact (reference variant): the reference's p_exact (:98-188) is a DP over
// dp_i[u] = sum_{k=0..n2} dp_{i-1}[u-k] in wrapping uint64 followed by sequential double
// sums. One table per distinct (n1, n2) holds pmf[u] = (double)dp[u] and the running
// double sums prefix[k] = prefix[k-1] + pmf[k] (the reference's own summation order), so
// each test is an O(1) lookup that reproduces the reference bit for bit.
// Exact (MWU-null variant): the true null distribution of U, f(u; m, n) =
// f(u - n; m - 1, n) + f(u; m, n - 1) (counts in double, all additions of positive terms),
// tail-summed from the left like scipy's _MWU.sf.
#pragma once
#include <cstdint>

#include "common.cuh"
#include "pvalue_math.cuh"

namespace hpdex {

// erfc table of this device (see pvalue_math.cuh), built by erfc_table_kernel
__device__ double g_erfc_table[kErfcPoints * kErfcTerms];

__global__ void erfc_table_kernel() {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kErfcPoints) return;
    const double x = (double)k / kErfcPerUnit;
    double* c = g_erfc_table + (size_t)k * kErfcTerms;
    const double E = 1.1283791670955126 * exp(-x * x);  // 2 / sqrt(pi) * exp(-x^2)
    c[0] = erfc(x);
    double hm1 = 0.0, h = 1.0, fact = 1.0, sign = 1.0;  // H_(n-1), n!, (-1)^(n-1)
    for (int n = 1; n < kErfcTerms; ++n) {
        fact *= n;
        c[n] = -E * sign * h / fact;
        const double hn = 2.0 * x * h - 2.0 * (n - 1) * hm1;  // H_n from H_(n-1), H_(n-2)
        hm1 = h;
        h = hn;
        sign = -sign;
    }
}

// Self-check: max relative / absolute difference of erfc_tab against the math library's erfc
// on n points spread over [-8, 27] (relative only where erfc >= 1e-300).
__global__ void erfc_check_kernel(long long n, unsigned long long* max_rel_bits,
                                  unsigned long long* max_abs_bits) {
    double mr = 0.0, ma = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double x = -8.0 + 35.0 * ((double)i + 0.5) / (double)n;
        const double a = erfc_tab(x, g_erfc_table), b = erfc(x);
        const double e = fabs(a - b);
        ma = fmax(ma, e);
        if (b >= 1e-300) mr = fmax(mr, e / b);
    }
    // non-negative doubles order like their bit patterns
    atomicMax(max_rel_bits, (unsigned long long)__double_as_longlong(mr));
    atomicMax(max_abs_bits, (unsigned long long)__double_as_longlong(ma));
}

// erfc_tab at given points (hpdex_selftest_erfc_values)
__global__ void erfc_values_kernel(const double* x, long long n, double* out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = erfc_tab(x[i], g_erfc_table);
}

// Self-check of the divisions by a known reciprocal (pvalue_math.cuh) against IEEE division
// (__ddiv_rn), bit for bit, on n generated cases; counts the mismatches. Case kinds (i % 4):
//   0  tie sums by N (N - 1): integers below 2^53 over N in [2, 2^24]
//   1  random doubles with exponents in [-60, 60]
//   2  quotients next to a rounding midpoint: a = RN((q + ulp(q)/2) b)
//   3  x / 12 for random doubles and integers
// Kinds 0-2 also check a / 12.
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {  // splitmix64
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ double rand_double(unsigned long long r, int emin, int span) {
    const long long e = 1023 + emin + (long long)((r >> 52) % (unsigned long long)span);
    return __longlong_as_double((long long)((unsigned long long)e << 52 | (r & 0xfffffffffffffull)));
}
__global__ void division_check_kernel(long long n, unsigned long long seed,
                                      unsigned long long* mismatches) {
    unsigned long long bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long r1 = mix64(seed ^ (unsigned long long)i * 4u);
        const unsigned long long r2 = mix64(r1 + 1u);
        const int kind = (int)(i & 3);
        double a, b;
        if (kind == 0) {
            a = (double)(r1 >> (11 + (r2 >> 58) % 53));  // integers of 1..53 bits
            const double N = (double)(2 + (long long)((r2 >> 20) % (1u << 24)));
            b = __dmul_rn(N, __dsub_rn(N, 1.0));
        } else if (kind == 1 || kind == 3) {
            a = rand_double(r1, -60, 121);
            b = rand_double(r2, -60, 121);
            if (kind == 3 && (r2 & 1u)) a = (double)(r1 >> 11);
        } else {
            const double q = rand_double(r1, -30, 61);
            b = rand_double(r2, -30, 61);
            const double half_ulp = __dsub_rn(__longlong_as_double(__double_as_longlong(q) + 1), q) * 0.5;
            a = __fma_rn(q, b, __dmul_rn(half_ulp, b));
        }
        if (kind != 3) {
            const double y = __drcp_rn(b);
            if (__double_as_longlong(div_by_recip(a, b, y)) != __double_as_longlong(__ddiv_rn(a, b))) ++bad;
        }
        if (__double_as_longlong(div12(a)) != __double_as_longlong(__ddiv_rn(a, 12.0))) ++bad;
    }
    if (bad) atomicAdd(mismatches, bad);
}

struct PArgs {
    const double* U1;
    double* P;                 // holds the (masked) tie sum on entry; P on exit unless P_out
    long long n;               // T * col_w: the tests of columns [col_lo, col_lo + col_w)
    int32_t n_cols;
    int32_t col_lo, col_w;
    double* U1_out;            // optional: U1 and P written here instead (same [T][n_cols]
    double* P_out;             //   layout; may be host memory the device can access)
    const long long* group_rows;
    const uint32_t* n1g;       // zero_handling = none: per gene
    const uint32_t* n2t;       // zero_handling = none: per test
    const PConst* pk;          // zero_handling min / max / mix: per target (or null)
    int32_t zero_handling;
    int32_t alternative;
    double cc;
    int32_t fast;              // fast_norm: the reference's fast normal tail (p_asymptotic_fast)
};

// test i of the column range -> its target t and column c, at idx = t * n_cols + c
__device__ __forceinline__ long long test_index(const PArgs& a, long long i, int& t, int& c) {
    t = (int)(i / a.col_w);
    c = a.col_lo + (int)(i - (long long)t * a.col_w);
    return (long long)t * a.n_cols + c;
}
__device__ __forceinline__ void test_sizes(const PArgs& a, int t, int c, long long idx, double& n1,
                                           double& n2) {
    if (a.zero_handling == ZH_NONE) {
        n1 = (double)a.n1g[c];
        n2 = (double)a.n2t[idx];
    } else {
        n1 = (double)a.group_rows[0];
        n2 = (double)a.group_rows[t + 1];
    }
}

// the p-value of test i of a's column range
__device__ __forceinline__ void pvalue_one(const PArgs& a, long long i) {
    int t, c;
    const long long idx = test_index(a, i, t, c);
    double n1, n2;
    test_sizes(a, t, c, idx, n1, n2);
    const double u1 = a.U1[idx];
    double p;
    if (a.fast) p = p_asymptotic_fast(u1, n1, n2, a.P[idx], a.cc, a.alternative);
    else if (a.pk && a.zero_handling != ZH_NONE)
        p = p_asymptotic_k(u1, a.pk[t], a.P[idx], a.cc, a.alternative, g_erfc_table);
    else p = p_asymptotic(u1, n1, n2, a.P[idx], a.cc, a.alternative, g_erfc_table);
    if (a.P_out) {
        a.U1_out[idx] = u1;
        a.P_out[idx] = p;
    } else {
        a.P[idx] = p;
    }
}

__global__ void mwu_pvalue_asymptotic_kernel(const PArgs a) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride)
        pvalue_one(a, i);
}

// The p-values of several independent test sets in one launch (a batch of the serving loop):
// set k covers the tests [first[k], first[k + 1]) of the launch.
__global__ void mwu_pvalue_batch_kernel(const PArgs* sets, const long long* first, int n_sets) {
    const long long n = first[n_sets];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        int lo = 0, hi = n_sets - 1;  // the last set k with first[k] <= i
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (first[mid] <= i) lo = mid; else hi = mid - 1;
        }
        pvalue_one(sets[lo], i - first[lo]);
    }
}

// ---------------- exact tables ----------------
struct ExactTables {
    const long long* pair_n1;     // [n_pairs]
    const long long* pair_n2;     // [n_pairs]
    const long long* offset;      // [n_pairs] start of each table in `tables`
    double* tables;               // per pair: pmf[0..n1*n2] then prefix[0..n1*n2]
    unsigned long long* work;     // uint64 scratch: 2 * (n1*n2 + 1) per pair (reference)
    const long long* work_off;    // [n_pairs]
    int32_t n_pairs;
    int32_t variant;              // 0 reference, 1 MWU null
};

// Reference variant: one CTA per (n1, n2). The sliding-window recurrence is a prefix-sum
// difference, computed here with a block-wide inclusive scan in wrapping uint64 (the same
// values mod 2^64 as the reference's sequential window), then the running double sums.
template <int NT>
__global__ void __launch_bounds__(NT) exact_reference_table_kernel(const ExactTables t) {
    __shared__ unsigned long long s_carry;
    __shared__ unsigned long long s_w[NT / 32];
    const int pi = blockIdx.x;
    if (pi >= t.n_pairs) return;
    const long long n1 = t.pair_n1[pi], n2 = t.pair_n2[pi];
    const long long umax = n1 * n2;
    unsigned long long* cur = t.work + t.work_off[pi];
    unsigned long long* pre = cur + (umax + 1);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (long long u = tid; u <= umax; u += NT) cur[u] = (u == 0) ? 1ull : 0ull;
    __syncthreads();
    for (long long i = 1; i <= n1; ++i) {
        const long long up = i * n2;
        // inclusive prefix sums of cur[0..up] (mod 2^64) into pre
        if (tid == 0) s_carry = 0ull;
        __syncthreads();
        for (long long base = 0; base <= up; base += NT) {
            const long long u = base + tid;
            unsigned long long v = (u <= up) ? cur[u] : 0ull;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long o = __shfl_up_sync(0xffffffffu, v, d);
                if (lane >= d) v += o;
            }
            if (lane == 31) s_w[warp] = v;
            __syncthreads();
            if (warp == 0) {
                unsigned long long w = lane < NT / 32 ? s_w[lane] : 0ull;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const unsigned long long o = __shfl_up_sync(0xffffffffu, w, d);
                    if (lane >= d) w += o;
                }
                if (lane < NT / 32) s_w[lane] = w;
            }
            __syncthreads();
            const unsigned long long before = s_carry + (warp ? s_w[warp - 1] : 0ull);
            if (u <= up) pre[u] = before + v;
            __syncthreads();
            if (tid == NT - 1) s_carry = before + v;
            __syncthreads();
        }
        // dp_i[u] = pre[u] - pre[u - n2 - 1]
        for (long long u = tid; u <= up; u += NT)
            cur[u] = pre[u] - ((u >= n2 + 1) ? pre[u - n2 - 1] : 0ull);
        __syncthreads();
    }
    // pmf and running double sums in the reference's order (sequential, one thread)
    double* pmf = t.tables + t.offset[pi];
    for (long long u = tid; u <= umax; u += NT) pmf[u] = (double)cur[u];
    __syncthreads();
    if (tid == 0) {
        double* pre = pmf + (umax + 1);
        double s = 0.0;
        for (long long u = 0; u <= umax; ++u) {
            s = __dadd_rn(s, pmf[u]);
            pre[u] = s;
        }
    }
}

// MWU-null variant: counts f(u; m, k) for k = 0..n (m = min side), built in place:
// the table for (m', k) is obtained from (m'-1, k) and (m', k-1). Memory: (m+1) rows of
// (m*n+1) doubles, held in `work` reinterpreted as double. One CTA per pair.
template <int NT>
__global__ void __launch_bounds__(NT) exact_null_table_kernel(const ExactTables t) {
    const int pi = blockIdx.x;
    if (pi >= t.n_pairs) return;
    long long m = t.pair_n1[pi], n = t.pair_n2[pi];
    if (m > n) { const long long s = m; m = n; n = s; }
    const long long umax = m * n;
    double* rows = reinterpret_cast<double*>(t.work + t.work_off[pi]);  // (m+1) x (umax+1)
    const long long W = umax + 1;
    const int tid = threadIdx.x;
    // k = 0 (no targets): f(u; m', 0) = [u == 0] for every m'
    for (long long j = tid; j < (m + 1) * W; j += NT) rows[j] = ((j % W) == 0) ? 1.0 : 0.0;
    __syncthreads();
    for (long long k = 1; k <= n; ++k) {
        // row m' for (m', k) = row m'-1 (already (m'-1, k)) shifted by k + row m' (m', k-1)
        for (long long mm = 1; mm <= m; ++mm) {
            double* r = rows + mm * W;
            const double* rp = rows + (mm - 1) * W;
            const long long top = mm * k;
            for (long long u = top - tid; u >= 0; u -= NT) {
                // descending u keeps r[u] (old, (mm, k-1)) unread-after-write safe per u
                const double add = (u >= k) ? rp[u - k] : 0.0;
                r[u] = __dadd_rn(r[u], add);
            }
            __syncthreads();
        }
    }
    const double* f = rows + m * W;
    double* pmf = t.tables + t.offset[pi];
    for (long long u = tid; u <= umax; u += NT) pmf[u] = f[u];
    __syncthreads();
    if (tid == 0) {
        double* pre = pmf + (umax + 1);
        double s = 0.0;
        for (long long u = 0; u <= umax; ++u) {
            s = __dadd_rn(s, pmf[u]);
            pre[u] = s;
        }
    }
}

struct ExactArgs {
    const double* U1;
    double* P;
    long long n;
    int32_t n_cols;
    const long long* group_rows;
    const uint32_t* n1g;
    const uint32_t* n2t;
    int32_t zero_handling;
    int32_t alternative;
    int32_t variant;
    // table lookup: pair index of the test's (n1, n2), via a dense map over (n1, n2) when
    // zero_handling != none (per target), else via per-test pair ids
    const int32_t* pair_of_target;  // [T]  (zero_handling != none)
    const int32_t* pair_of_test;    // [T * n_cols] (zero_handling = none, host-built map)
    const int32_t* pair_index;      // zero_handling = none: pair of (n1, n2) at n1 * pair_w + n2
    int32_t pair_w;                 //   (when non-null; built from exact_mark_pairs_kernel)
    int32_t pair_h;
    const long long* pair_n1;
    const long long* pair_n2;
    const long long* offset;
    const double* tables;
    const double* recip;            // [n_pairs] RN(1 / total) of each table, 0 where the
                                    // quotients must take an IEEE division (total 0 or not finite)
};

// RN(1 / total) of each table (total = prefix[n1*n2]), for its quotients by the total: the
// numerators are counts (0 or at least 1), so with 1 <= total < 2^960 no quotient leaves the
// normal range and Markstein's division (div_by_recip) gives the IEEE quotient. A total of 0 (the
// reference variant's wrapping counts) or beyond keeps the IEEE division.
__global__ void exact_recip_kernel(const long long* pair_n1, const long long* pair_n2,
                                   const long long* offset, const double* tables, int32_t n_pairs,
                                   double* recip) {
    for (int pi = blockIdx.x * blockDim.x + threadIdx.x; pi < n_pairs; pi += gridDim.x * blockDim.x) {
        const long long umax = pair_n1[pi] * pair_n2[pi];
        const double total = tables[offset[pi] + 2 * umax + 1];
        recip[pi] = (total >= 1.0 && total < 0x1p960) ? __drcp_rn(total) : 0.0;
    }
}

// survival P(U >= floor(U)) from a table, the reference's formula (:160-179); y = RN(1 / total)
// or 0 (IEEE division)
__device__ __forceinline__ double table_sf(const double* pmf, long long umax, double U, double y) {
    if (umax == 0) return 1.0;
    const double* pre = pmf + (umax + 1);
    double Uc = U < 0.0 ? 0.0 : U;
    if (Uc > (double)umax) Uc = (double)umax;
    const long long u_stat = (long long)floor(Uc);
    const double total = pre[umax];
    const long long kc = umax - u_stat;
    const long long small = u_stat < kc ? u_stat : kc;
    const double cdf_small = pre[small];
    const double pmf_small = pmf[small];
    auto quot = [&](double x) { return y != 0.0 ? div_by_recip(x, total, y) : __ddiv_rn(x, total); };
    if (u_stat <= kc)
        return __dadd_rn(__dsub_rn(1.0, quot(cdf_small)), quot(pmf_small));
    return quot(cdf_small);
}

// zero_handling none: marks the (n1, n2) cells of a dense H x W map that occur among the tests
// (sample sizes outside the map only come with duplicate row ids, which the run reports). Few
// cells are marked by many tests: a test stores only while its cell still reads 0, so the stores
// to one cell do not queue up (every store writes the same 1).
__global__ void exact_mark_pairs_kernel(const uint32_t* n1g, const uint32_t* n2t, long long n,
                                        int32_t n_cols, int32_t H, int32_t W, unsigned char* mark) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t n1 = n1g[i % n_cols], n2 = n2t[i];
        if (n1 < (uint32_t)H && n2 < (uint32_t)W) {
            unsigned char* m = mark + (size_t)n1 * W + n2;
            if (__ldcg(m) == 0) *m = 1;
        }
    }
}

__global__ void mwu_pvalue_exact_kernel(const ExactArgs a) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const int t = (int)(i / a.n_cols);
        int pi;
        if (a.zero_handling != ZH_NONE) {
            pi = a.pair_of_target[t];
        } else if (a.pair_index) {
            const uint32_t n1 = a.n1g[i % a.n_cols], n2 = a.n2t[i];
            pi = (n1 < (uint32_t)a.pair_h && n2 < (uint32_t)a.pair_w)
                     ? a.pair_index[(size_t)n1 * a.pair_w + n2] : -1;
        } else {
            pi = a.pair_of_test[i];
        }
        const double U1 = a.U1[i];
        double p = 1.0;
        if (pi >= 0) {
            const long long n1 = a.pair_n1[pi], n2 = a.pair_n2[pi];
            const double nprod = __dmul_rn((double)n1, (double)n2);
            const double* pmf = a.tables + a.offset[pi];
            const long long umax = n1 * n2;
            double U;
            if (a.alternative == ALT_TWO_SIDED) {
                const double U2 = __dsub_rn(nprod, U1);
                U = U1 > U2 ? U1 : U2;
            } else if (a.alternative == ALT_GREATER) {
                U = U1;
            } else {
                U = __dsub_rn(nprod, U1);
            }
            const double sf = table_sf(pmf, umax, U, a.recip[pi]);
            p = (a.alternative == ALT_TWO_SIDED) ? __dmul_rn(2.0, sf) : sf;
            if (p < 0.0) p = 0.0;
            if (p > 1.0) p = 1.0;
        }
        a.P[i] = p;
    }
}

}  // namespace hpdex
