/*
 * mwu_oracle.c -- CPU restatement of hpdex's Mann-Whitney U backend.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle for the GPU path and the
 * "port" CPU baseline timed by bench.py. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU legs load it; the hpdex_gb300 product never links or calls it.
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own C++ kernel (built
 * from its unmodified sources with oracle/build_ref.sh) on seeded inputs, and
 * tests/test_oracle.py checks this restatement against every one of them.
 *
 * It follows the reference algorithm step by step (same complexity, same double
 * arithmetic), citing AI4Cell/hpdex src/cpp/mannwhitneyu.cpp:
 *   - gather valid entries per group              :914-926
 *   - sort each group slice                      :929-932
 *   - zero handling none / min,max / mix         :935-1039
 *   - two-pointer merge with midranks and ties   :618-659, :791-840
 *   - zero block at head or tail                 :728-788
 *   - zero block in the middle                   :662-725
 *   - precise asymptotic p (erfc)                :15-96
 *   - exact p (bounded-composition DP, uint64)   :98-188, :243-282
 *   - group_mean and its Kahan variant           :1118-1192, :1195-1272
 * Errors reproduce the single-threaded reference: the lowest failing column wins,
 * and within it the reference group is checked before targets 1..T.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { DT_I8 = 0, DT_U8, DT_I16, DT_U16, DT_I32, DT_U32, DT_I64, DT_U64, DT_F32, DT_F64 };
enum { ZH_NONE = 0, ZH_MIN = 1, ZH_MAX = 2, ZH_MIX = 3 };
enum { ALT_LESS = 0, ALT_GREATER = 1, ALT_TWO_SIDED = 2 };
enum { METHOD_EXACT = 1, METHOD_ASYMPTOTIC = 2 };

/* value p of the CSC data array, cast to double as mannwhitneyu.cpp:920 does */
static inline double load_value(int dtype, const void* data, int64_t p) {
    switch (dtype) {
    case DT_I8:  return (double)((const int8_t*)data)[p];
    case DT_U8:  return (double)((const uint8_t*)data)[p];
    case DT_I16: return (double)((const int16_t*)data)[p];
    case DT_U16: return (double)((const uint16_t*)data)[p];
    case DT_I32: return (double)((const int32_t*)data)[p];
    case DT_U32: return (double)((const uint32_t*)data)[p];
    case DT_I64: return (double)((const int64_t*)data)[p];
    case DT_U64: return (double)((const uint64_t*)data)[p];
    case DT_F32: return (double)((const float*)data)[p];
    default:     return ((const double*)data)[p];
    }
}

/* is_valid_value (mannwhitneyu.cpp:611-615) sees the double, so only NaN/Inf fail */
static inline int valid_value(double v) { return isfinite(v); }

/* ---------------- sort of a double slice (stands in for VQSortStatic) ---------------- */
static void insertion_sort(double* a, int64_t n) {
    for (int64_t i = 1; i < n; ++i) {
        double x = a[i];
        int64_t j = i - 1;
        while (j >= 0 && a[j] > x) { a[j + 1] = a[j]; --j; }
        a[j + 1] = x;
    }
}

static void sort_doubles(double* a, int64_t n) {
    /* introsort-free quicksort with median-of-three and an explicit stack */
    int64_t stack_lo[128], stack_hi[128];
    int sp = 0;
    stack_lo[sp] = 0; stack_hi[sp] = n - 1; ++sp;
    while (sp > 0) {
        --sp;
        int64_t lo = stack_lo[sp], hi = stack_hi[sp];
        while (hi - lo > 24) {
            int64_t mid = lo + (hi - lo) / 2;
            double x = a[lo], y = a[mid], z = a[hi];
            double piv = (x < y) ? ((y < z) ? y : ((x < z) ? z : x)) : ((x < z) ? x : ((y < z) ? z : y));
            int64_t i = lo, j = hi;
            while (i <= j) {
                while (a[i] < piv) ++i;
                while (piv < a[j]) --j;
                if (i <= j) { double t = a[i]; a[i] = a[j]; a[j] = t; ++i; --j; }
            }
            /* recurse into the smaller side first (push the larger) */
            if (j - lo < hi - i) {
                if (i < hi) { stack_lo[sp] = i; stack_hi[sp] = hi; ++sp; }
                hi = j;
            } else {
                if (lo < j) { stack_lo[sp] = lo; stack_hi[sp] = j; ++sp; }
                lo = i;
            }
        }
        insertion_sort(a + lo, hi - lo + 1);
    }
}

/* ---------------- merge of two sorted runs (mannwhitneyu.cpp:618-659) ---------------- */
/* Walks the union of a[0..na) and b[0..nb) in ascending order, giving each tie block the
 * midrank of its global rank interval starting at `rank`. Adds the a-side ranks to *R1 and
 * t^3 - t of each tie block to *tie; returns the next free rank. */
static int64_t merge_segment(const double* a, int64_t na, const double* b, int64_t nb,
                             int64_t rank, double* R1, double* tie) {
    int64_t i = 0, j = 0;
    while (i < na || j < nb) {
        double v;
        if (i < na && (j >= nb || !(b[j] < a[i]))) v = a[i];
        else v = b[j];
        int64_t ea = 0, eb = 0;
        while (i + ea < na && !(a[i + ea] < v) && !(v < a[i + ea])) ++ea;
        while (j + eb < nb && !(b[j + eb] < v) && !(v < b[j + eb])) ++eb;
        const int64_t t = ea + eb;
        const double start = (double)rank;
        const double end = (double)(rank + t - 1);
        *R1 += (double)ea * (0.5 * (start + end));
        if (t > 1) {
            const double tt = (double)t;
            *tie += tt * tt * tt - tt;
        }
        rank += t;
        i += ea;
        j += eb;
    }
    return rank;
}

/* splits a sorted slice into negatives, explicit zeros, positives */
static void split_signs(const double* a, int64_t n, int64_t* neg_end, int64_t* zero_end) {
    int64_t i = 0;
    while (i < n && a[i] < 0.0) ++i;
    *neg_end = i;
    while (i < n && !(0.0 < a[i]) && !(a[i] < 0.0)) ++i;
    *zero_end = i;
}

/* zero block of `ref_z + tar_z` tied entries placed at rank interval starting at `rank` */
static int64_t emit_zero_block(int64_t ref_z, int64_t tar_z, int64_t rank, double* R1, double* tie) {
    const int64_t t = ref_z + tar_z;
    if (t > 0) {
        const double start = (double)rank, end = (double)(rank + t - 1);
        *R1 += (double)ref_z * (0.5 * (start + end));
        if (t > 1) { const double tt = (double)t; *tie += tt * tt * tt - tt; }
        rank += t;
    }
    return rank;
}

/* mode min / max: mannwhitneyu.cpp:728-788; mode mix: :662-725; mode none: :791-840 */
static void rank_sum(int zero_handling, const double* a, int64_t na, const double* b, int64_t nb,
                     int64_t a_zero_implicit, int64_t b_zero_implicit, double* R1, double* tie) {
    *R1 = 0.0;
    *tie = 0.0;
    if (zero_handling == ZH_NONE) {
        merge_segment(a, na, b, nb, 1, R1, tie);
        return;
    }
    int64_t an, az, bn, bz;
    split_signs(a, na, &an, &az);
    split_signs(b, nb, &bn, &bz);
    const int64_t A0 = (az - an) + a_zero_implicit;
    const int64_t B0 = (bz - bn) + b_zero_implicit;
    int64_t rank = 1;
    if (zero_handling == ZH_MIX) {
        rank = merge_segment(a, an, b, bn, rank, R1, tie);
        rank = emit_zero_block(A0, B0, rank, R1, tie);
        merge_segment(a + az, na - az, b + bz, nb - bz, rank, R1, tie);
        return;
    }
    if (zero_handling == ZH_MIN) rank = emit_zero_block(A0, B0, rank, R1, tie);
    rank = merge_segment(a, an, b, bn, rank, R1, tie);
    rank = merge_segment(a + az, na - az, b + bz, nb - bz, rank, R1, tie);
    if (zero_handling == ZH_MAX) emit_zero_block(A0, B0, rank, R1, tie);
}

/* ---------------- p-values ---------------- */
#ifndef M_SQRT1_2
#define M_SQRT1_2 0.70710678118654752440
#endif

/* compute_mu_sigma_precise (mannwhitneyu.cpp:24-37), same operation order */
static inline void mu_sigma(double n1, double n2, double tie_sum, double* mu, double* sigma) {
    const double N = n1 + n2;
    const double nm = n1 * n2;
    *mu = 0.5 * nm;
    double tie_term = 0.0;
    const double denom = N * (N - 1.0);
    if (denom > 0.0) tie_term = tie_sum / denom;
    const double var = nm * ((N + 1.0) - tie_term) / 12.0;
    *sigma = (var > 0.0) ? sqrt(var) : 0.0;
}

static inline double norm_sf(double z) { return 0.5 * erfc(z * M_SQRT1_2); }

/* array_p_asymptotic_{greater,less,two_sided}_precise (mannwhitneyu.cpp:39-96) */
double oracle_p_asymptotic(double U1, double n1, double n2, double tie_sum, double cc, int alternative) {
    double mu, sigma, p = 1.0;
    mu_sigma(n1, n2, tie_sum, &mu, &sigma);
    if (alternative == ALT_TWO_SIDED) {
        const double nm = n1 * n2;
        const double U2 = nm - U1;
        const double U = (U1 > U2 ? U1 : U2);
        if (sigma > 0.0) {
            const double z = (U - mu - cc) / sigma;
            p = 2.0 * norm_sf(z);
            if (p > 1.0) p = 1.0;
            if (p < 0.0) p = 0.0;
        }
        return p;
    }
    double U = U1;
    if (alternative == ALT_LESS) U = n1 * n2 - U1;
    if (sigma > 0.0) {
        const double z = (U - mu - cc) / sigma;
        p = norm_sf(z);
    }
    return (p < 0.0 ? 0.0 : (p > 1.0 ? 1.0 : p));
}

/* fast_norm path (src/cpp/include/common.hpp:14-92, scalar form): Numerical Recipes' erfcc
 * Chebyshev fit with libm exp; mu and 1/sigma as precompute_mu_inv_sd; two-sided
 * z = (|U1 - mu| - cc) / sigma, greater (U1 - mu - cc) / sigma, less (U1 - mu + cc) / sigma
 * with p = 1 - sf. */
static double erfcc_nr(double x) {
    const double ax = fabs(x);
    const double t = 1.0 / (1.0 + 0.5 * ax);
    const double tau = t * exp(-ax * ax - 1.26551223 +
                               t * (1.00002368 + t * (0.37409196 + t * (0.09678418 +
                               t * (-0.18628806 + t * (0.27886807 + t * (-1.13520398 +
                               t * (1.48851587 + t * (-0.82215223 + t * 0.17087277)))))))));
    double r = (x >= 0.0) ? tau : 2.0 - tau;
    return r < 0.0 ? 0.0 : (r > 2.0 ? 2.0 : r);
}

double oracle_p_asymptotic_fast(double U1, double n1, double n2, double tie_sum, double cc, int alternative) {
    const double N = n1 + n2;
    const double mu = 0.5 * n1 * n2;
    const double denom = N * (N - 1.0);
    const double base = n1 * n2 / 12.0;
    const double var = (denom > 0.0) ? base * (N + 1.0 - tie_sum / denom) : n1 * n2 * (N + 1.0) / 12.0;
    const double inv_sd = (var <= 0.0) ? 0.0 : 1.0 / sqrt(var);
    if (inv_sd == 0.0) return 1.0;
    const double s2 = sqrt(2.0);
    if (alternative == ALT_TWO_SIDED) return 2.0 * (0.5 * erfcc_nr(((fabs(U1 - mu) - cc) * inv_sd) / s2));
    if (alternative == ALT_GREATER) return 0.5 * erfcc_nr(((U1 - mu - cc) * inv_sd) / s2);
    return 1.0 - 0.5 * erfcc_nr(((U1 - mu + cc) * inv_sd) / s2);
}

void oracle_p_asymptotic_fast_array(const double* U1, const double* n1, const double* n2,
                                    const double* tie_sum, double cc, int alternative, int64_t n,
                                    double* out) {
    for (int64_t i = 0; i < n; ++i)
        out[i] = oracle_p_asymptotic_fast(U1[i], n1[i], n2[i], tie_sum[i], cc, alternative);
}

/* p_exact (mannwhitneyu.cpp:98-188): the reference's counting DP. Its recurrence
 * dp_i[u] = sum_{k=0..n2} dp_{i-1}[u-k], applied n1 times, counts compositions of u
 * into n1 parts in [0, n2] (not the MWU null), in uint64 arithmetic that wraps. The
 * tail uses sequential double sums over u = 0.. and the symmetry switch of :172-179. */
double oracle_p_exact_reference(double U, int64_t n1, int64_t n2) {
    const int64_t Umax = n1 * n2;
    if (Umax == 0) return 1.0;
    double Uc = U < 0.0 ? 0.0 : U;
    if (Uc > (double)Umax) Uc = (double)Umax;
    const int64_t u_stat = (int64_t)floor(Uc);
    uint64_t* cur = (uint64_t*)calloc((size_t)Umax + 1, sizeof(uint64_t));
    uint64_t* nxt = (uint64_t*)calloc((size_t)Umax + 1, sizeof(uint64_t));
    cur[0] = 1;
    for (int64_t i = 1; i <= n1; ++i) {
        const int64_t up = i * n2;
        uint64_t win = 0;
        for (int64_t u = 0; u <= up; ++u) {
            if (u <= (i - 1) * n2) win += cur[u];
            if (u >= n2 + 1) win -= cur[u - (n2 + 1)];
            nxt[u] = win;
        }
        uint64_t* t = cur; cur = nxt; nxt = t;
        memset(nxt, 0, sizeof(uint64_t) * ((size_t)Umax + 1));
    }
    double total = 0.0;
    for (int64_t u = 0; u <= Umax; ++u) total += (double)cur[u];
    const int64_t kc = Umax - u_stat;
    const int64_t small = u_stat < kc ? u_stat : kc;
    double cdf_small = 0.0;
    for (int64_t u = 0; u <= small; ++u) cdf_small += (double)cur[u];
    const double pmf_small = (double)cur[small];
    double sf;
    if (u_stat <= kc) sf = 1.0 - cdf_small / total + pmf_small / total;
    else sf = cdf_small / total;
    free(cur);
    free(nxt);
    return sf;
}

/* p_exact_parallel body (mannwhitneyu.cpp:243-282) */
double oracle_p_exact_alt(double U1, double n1, double n2, int alternative) {
    const int64_t a = (int64_t)n1, b = (int64_t)n2;
    const double nprod = (double)a * (double)b;
    double p = 1.0;
    if (alternative == ALT_TWO_SIDED) {
        const double U2 = nprod - U1;
        p = 2.0 * oracle_p_exact_reference(U1 > U2 ? U1 : U2, a, b);
    } else if (alternative == ALT_GREATER) {
        p = oracle_p_exact_reference(U1, a, b);
    } else {
        p = oracle_p_exact_reference(nprod - U1, a, b);
    }
    if (p < 0.0) p = 0.0;
    if (p > 1.0) p = 1.0;
    return p;
}

/* ---------------- the MWU driver (mannwhitneyu.cpp:843-1065) ---------------- */
static void set_err(char* err, int errlen, const char* msg) {
    if (err && errlen > 0) { strncpy(err, msg, (size_t)errlen - 1); err[errlen - 1] = 0; }
}

/* Outputs are gene-major like the reference: index = gene * n_targets + (g - 1).
 * Returns 0 on success, 1 on a reference-style runtime error (message in err). */
int oracle_mwu(int dtype, const void* data, const int64_t* indices, const int64_t* indptr,
               int64_t R, int64_t C, const int32_t* group_id, int64_t n_targets,
               int ref_sorted, int tar_sorted, int tie_correction, int use_continuity,
               int zero_handling, int alternative, int method, int threads,
               double* U1_out, double* P_out, char* err, int errlen) {
    (void)ref_sorted; (void)tar_sorted; /* slices are always sorted (the flags only skip work) */
    if (n_targets < 1) { set_err(err, errlen, "[mannwhitney] n_targets must be >= 1 (>=1 target groups)"); return 1; }
    const int64_t G = n_targets + 1;
    const int64_t npairs = C * n_targets;
    const double tie_mask = tie_correction ? 1.0 : 0.0;
    const double cc = use_continuity ? 0.5 : 0.0;

    int64_t* group_rows = (int64_t*)calloc((size_t)G, sizeof(int64_t));
    int64_t* group_off = (int64_t*)calloc((size_t)G + 1, sizeof(int64_t));
    for (int64_t r = 0; r < R; ++r) {
        const int g = group_id[r];
        if (g >= 0 && g < G) ++group_rows[g];
    }
    for (int64_t g = 0; g < G; ++g) group_off[g + 1] = group_off[g] + group_rows[g];
    const int64_t cap = group_off[G];

    double* n1_arr = (double*)calloc((size_t)(npairs > 0 ? npairs : 1), sizeof(double));
    double* n2_arr = (double*)calloc((size_t)(npairs > 0 ? npairs : 1), sizeof(double));
    double* tie_arr = (double*)calloc((size_t)(npairs > 0 ? npairs : 1), sizeof(double));
    /* per column: 0 = ok, else 1 + failing group (0 = reference) */
    int64_t* col_err = (int64_t*)calloc((size_t)(C > 0 ? C : 1), sizeof(int64_t));
    for (int64_t i = 0; i < npairs; ++i) { U1_out[i] = 0.0; P_out[i] = 1.0; }

#ifdef _OPENMP
    if (threads < 1) threads = omp_get_max_threads();
    #pragma omp parallel num_threads(threads)
#endif
    {
        double* buf = (double*)malloc(sizeof(double) * (size_t)(cap > 0 ? cap : 1));
        int64_t* cnt = (int64_t*)malloc(sizeof(int64_t) * (size_t)G);
#ifdef _OPENMP
        #pragma omp for schedule(static)
#endif
        for (int64_t c = 0; c < C; ++c) {
            memset(cnt, 0, sizeof(int64_t) * (size_t)G);
            for (int64_t p = indptr[c]; p < indptr[c + 1]; ++p) {
                const int64_t r = indices[p];
                if (r < 0 || r >= R) continue;
                const int g = group_id[r];
                if (g < 0 || g >= G) continue;
                const double v = load_value(dtype, data, p);
                if (!valid_value(v)) continue;
                buf[group_off[g] + cnt[g]] = v;
                ++cnt[g];
            }
            for (int64_t g = 0; g < G; ++g)
                if (cnt[g] > 1) sort_doubles(buf + group_off[g], cnt[g]);

            const int64_t n1 = (zero_handling == ZH_NONE) ? cnt[0] : group_rows[0];
            if (n1 < 2) { col_err[c] = 1; continue; }
            for (int64_t g = 1; g < G; ++g) {
                const int64_t n2 = (zero_handling == ZH_NONE) ? cnt[g] : group_rows[g];
                if (n2 < 2) { if (!col_err[c]) col_err[c] = 1 + g; continue; }
                double R1, tie;
                rank_sum(zero_handling, buf, cnt[0], buf + group_off[g], cnt[g],
                         group_rows[0] - cnt[0], group_rows[g] - cnt[g], &R1, &tie);
                const double n1d = (double)n1;
                const int64_t idx = c * n_targets + (g - 1);
                U1_out[idx] = R1 - n1d * (n1d + 1.0) * 0.5;
                n1_arr[idx] = n1d;
                n2_arr[idx] = (double)n2;
                tie_arr[idx] = tie * tie_mask;
            }
        }
        free(buf);
        free(cnt);
    }

    int status = 0;
    for (int64_t c = 0; c < C; ++c) {
        if (col_err[c]) {
            char msg[160];
            if (col_err[c] == 1) snprintf(msg, sizeof msg, "Sample too small for reference at column %lld", (long long)c);
            else snprintf(msg, sizeof msg, "Sample too small for group %lld at column %lld", (long long)(col_err[c] - 1), (long long)c);
            set_err(err, errlen, msg);
            status = 1;
            break;
        }
    }
    if (status == 0) {
#ifdef _OPENMP
        #pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
#endif
        for (int64_t i = 0; i < npairs; ++i) {
            if (method == METHOD_ASYMPTOTIC)
                P_out[i] = oracle_p_asymptotic(U1_out[i], n1_arr[i], n2_arr[i], tie_arr[i], cc, alternative);
            else
                P_out[i] = oracle_p_exact_alt(U1_out[i], n1_arr[i], n2_arr[i], alternative);
        }
    }
    free(group_rows); free(group_off); free(n1_arr); free(n2_arr); free(tie_arr); free(col_err);
    return status;
}

/* Per-pair statistics before the p-value stage (same indexing as U1_out); used by the
 * tests to check tie sums and group sizes independently of erfc. */
int oracle_mwu_stats(int dtype, const void* data, const int64_t* indices, const int64_t* indptr,
                     int64_t R, int64_t C, const int32_t* group_id, int64_t n_targets,
                     int zero_handling, double* U1_out, double* n1_out, double* n2_out,
                     double* tie_out) {
    const int64_t G = n_targets + 1;
    int64_t* group_rows = (int64_t*)calloc((size_t)G, sizeof(int64_t));
    int64_t* group_off = (int64_t*)calloc((size_t)G + 1, sizeof(int64_t));
    for (int64_t r = 0; r < R; ++r) {
        const int g = group_id[r];
        if (g >= 0 && g < G) ++group_rows[g];
    }
    for (int64_t g = 0; g < G; ++g) group_off[g + 1] = group_off[g] + group_rows[g];
    double* buf = (double*)malloc(sizeof(double) * (size_t)(group_off[G] > 0 ? group_off[G] : 1));
    int64_t* cnt = (int64_t*)malloc(sizeof(int64_t) * (size_t)G);
    for (int64_t c = 0; c < C; ++c) {
        memset(cnt, 0, sizeof(int64_t) * (size_t)G);
        for (int64_t p = indptr[c]; p < indptr[c + 1]; ++p) {
            const int64_t r = indices[p];
            if (r < 0 || r >= R) continue;
            const int g = group_id[r];
            if (g < 0 || g >= G) continue;
            const double v = load_value(dtype, data, p);
            if (!valid_value(v)) continue;
            buf[group_off[g] + cnt[g]] = v;
            ++cnt[g];
        }
        for (int64_t g = 0; g < G; ++g)
            if (cnt[g] > 1) sort_doubles(buf + group_off[g], cnt[g]);
        for (int64_t g = 1; g < G; ++g) {
            double R1, tie;
            rank_sum(zero_handling, buf, cnt[0], buf + group_off[g], cnt[g],
                     group_rows[0] - cnt[0], group_rows[g] - cnt[g], &R1, &tie);
            const double n1 = (double)((zero_handling == ZH_NONE) ? cnt[0] : group_rows[0]);
            const int64_t idx = c * n_targets + (g - 1);
            U1_out[idx] = R1 - n1 * (n1 + 1.0) * 0.5;
            n1_out[idx] = n1;
            n2_out[idx] = (double)((zero_handling == ZH_NONE) ? cnt[g] : group_rows[g]);
            tie_out[idx] = tie;
        }
    }
    free(buf); free(cnt); free(group_rows); free(group_off);
    return 0;
}

/* ---------------- group_mean (mannwhitneyu.cpp:1118-1192, Kahan :1195-1272) ---------------- */
/* Output is flat [gene * n_groups + g] like the reference. */
int oracle_group_mean(int dtype, const void* data, const int64_t* indices, const int64_t* indptr,
                      int64_t R, int64_t C, const int32_t* group_id, int64_t n_groups,
                      int include_zeros, int use_kahan, int threads, double* out) {
    const int64_t G = n_groups;
    if (G <= 0 || C <= 0) return 0;
    int64_t* group_rows = (int64_t*)calloc((size_t)G, sizeof(int64_t));
    for (int64_t r = 0; r < R; ++r) {
        const int g = group_id[r];
        if (g >= 0 && g < G) ++group_rows[g];
    }
#ifdef _OPENMP
    if (threads < 1) threads = omp_get_max_threads();
    #pragma omp parallel num_threads(threads)
#endif
    {
        double* sum = (double*)malloc(sizeof(double) * (size_t)G);
        double* comp = (double*)malloc(sizeof(double) * (size_t)G);
        int64_t* valid = (int64_t*)malloc(sizeof(int64_t) * (size_t)G);
        int64_t* invalid = (int64_t*)malloc(sizeof(int64_t) * (size_t)G);
#ifdef _OPENMP
        #pragma omp for schedule(dynamic)
#endif
        for (int64_t c = 0; c < C; ++c) {
            for (int64_t g = 0; g < G; ++g) { sum[g] = 0.0; comp[g] = 0.0; valid[g] = 0; invalid[g] = 0; }
            for (int64_t p = indptr[c]; p < indptr[c + 1]; ++p) {
                const int64_t r = indices[p];
                if (r < 0 || r >= R) continue;
                const int g = group_id[r];
                if (g < 0 || g >= G) continue;
                const double v = load_value(dtype, data, p);
                if (valid_value(v)) {
                    if (use_kahan) {
                        const double y = v - comp[g];
                        const double t = sum[g] + y;
                        comp[g] = (t - sum[g]) - y;
                        sum[g] = t;
                    } else {
                        sum[g] += v;
                    }
                    ++valid[g];
                } else {
                    ++invalid[g];
                }
            }
            for (int64_t g = 0; g < G; ++g) {
                const int64_t denom = include_zeros ? (group_rows[g] - invalid[g]) : valid[g];
                out[c * G + g] = (denom > 0) ? (sum[g] / (double)denom) : 0.0;
            }
        }
        free(sum); free(comp); free(valid); free(invalid);
    }
    free(group_rows);
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
