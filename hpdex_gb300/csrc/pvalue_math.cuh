// pvalue_math.cuh -- per-test p-value arithmetic of the MWU backend (sm_103a), shared by the
// p-value kernel and the rank kernel's fused p-value stage.
//
// Asymptotic: restates the reference's precise path (AI4Cell/hpdex src/cpp/mannwhitneyu.cpp
// :15-96) with the same double operation order. Every multiply / add / divide / sqrt is an
// explicitly round-to-nearest intrinsic so that no multiply-add is fused and z is the same
// double the reference computes, whatever the surrounding code. erfc is evaluated from a
// table (erfc_tab below): FP64 is the scarce pipe on GB300, and the table's Taylor step costs
// about a tenth of a library erfc, within a few ulp of it.
#pragma once
#include <cstdint>

#include "common.cuh"

namespace hpdex {

// ---------------------------------------------------------------------------------------
// erfc from a table. erfc is tabulated with its Taylor coefficients at x_k = k / 128,
// 0 <= x_k < 26.5; for x near x_k, erfc(x_k + d) = sum_n c_n(x_k) d^n with
//     c_0 = erfc(x_k),   c_n = -(2/sqrt(pi)) exp(-x_k^2) (-1)^(n-1) H_(n-1)(x_k) / n!,
// from erfc'(x) = -(2/sqrt(pi)) exp(-x^2) and d^m/dx^m exp(-x^2) = (-1)^m H_m(x) exp(-x^2),
// with the physicists' Hermite polynomials H_0 = 1, H_1 = 2x, H_(m+1) = 2x H_m - 2m H_(m-1).
// With |d| <= 1/256 the n-th term is about (2 x d)^n / n! of c_0, so 13 terms leave a
// truncation below 1e-17 relative up to x = 26.5. The sum runs as a Horner polynomial in d;
// erfc(x_k + d) / erfc(x_k) stays above exp(-0.21), so nothing cancels. The table is built
// once per device from the CUDA math library's erfc and exp. From 26.5 on (erfc below
// 2.3e-307, subnormal from x = 26.55, zero beyond x = 27.23) erfc_tail below takes over;
// for x < 0, erfc(x) = 2 - erfc(-x).
// ---------------------------------------------------------------------------------------
constexpr int kErfcPerUnit = 128;
constexpr int kErfcTerms = 13;
constexpr double kErfcXMax = 26.5;
constexpr int kErfcPoints = (int)(kErfcXMax * kErfcPerUnit) + 2;

// ---------------------------------------------------------------------------------------
// The deep tail, x >= 26.5, where the reference's p-values are tiny normal or subnormal
// doubles. The reference calls the host C library's erfc (glibc), which for large x forms
//     erfc(x) = RN( RN( exp(a) * F ) / x ),   a = -z^2 - 0.5625,   z = x with the low 32 bits
// of its encoding cleared (so z^2 and a are exact), and F, a second exponential, within a few
// ulp of erfc(x) x exp(-a). Once the result is near or below the smallest normal double, the
// roundings of exp(a), of the product and of the quotient onto the subnormal grid decide its
// value (the grid spacing, 4.9e-324, is far coarser than the error of F), so they are repeated
// here in that order, with F to about 1e-19:
//   exp(a) = 2^k exp(r), r = a - k ln 2 with ln 2 split in two (Cody and Waite: the high part
//            has 40 significant bits, so k times it is exact); exp(r) from the math library,
//            scaled by 2^(k+64) (exact) and by 2^-64, the one rounding onto the grid;
//   F      = K (1 + q)(1 + p), K = exp(0.5625) / sqrt(pi) as a double-double constant;
//            1 + q = x sqrt(pi) exp(x^2) erfc(x) from its asymptotic series
//            sum_n (-1)^n (2n-1)!! / (2x^2)^n (Abramowitz and Stegun 7.1.23; 8 terms leave less
//            than 2e-21 for x >= 26.5), and 1 + p = exp(-(x - z)(x + z)) from its Taylor series
//            (the exponent is below 8.4e-4); q and p are each below 1e-3, so their rounding
//            errors stay near 1e-19 of F;
//   exp(a) F is formed at a 2^64 scale (exact product split by an fma) and rounded once onto
//            the grid.
// A host restatement of these steps equals glibc's erfc on every one of 100,000 random points
// of [26.5, 27.3] whose value is below 1e-311; above it (the grid approaches full double
// precision) it differs on 1.4% of the points by one grid step, at most 4.8e-13 relative:
// glibc's own error in F.
// ---------------------------------------------------------------------------------------
static __device__ __noinline__ double erfc_tail(double ax) {
    const double z = __hiloint2double(__double2hiint(ax), 0);
    const double a = __dsub_rn(__dmul_rn(-z, z), 0.5625);  // exact
    // exp(a) < 2e-326 rounds to 0 (and below -750, 2^(k+64) would leave the normal range); NaN
    // stays NaN, as in the library
    if (!(a >= -750.0)) return a != a ? a : 0.0;
    const double ln2_hi = 0x1.62e42fefa4000p-1;    // ln 2 to 40 bits
    const double ln2_lo = -0x1.8432a1b0e2634p-43;  // RN(ln 2 - ln2_hi)
    const int k = __double2int_rn(__dmul_rn(a, 1.4426950408889634));  // ~ a / ln 2
    const double r = __dsub_rn(__fma_rn(-(double)k, ln2_hi, a), __dmul_rn((double)k, ln2_lo));
    const double s1 = __hiloint2double((k + 64 + 1023) << 20, 0);  // 2^(k+64), normal
    const double e1 = __dmul_rn(__dmul_rn(exp(r), s1), 0x1p-64);   // on the grid
    // 1 + q: the asymptotic series in u = 1 / (2 x^2), Horner from the 8th term down
    const double u = __ddiv_rn(0.5, __dmul_rn(ax, ax));
    double h = __fma_rn(-15.0, u, 1.0);
#pragma unroll
    for (int n = 13; n >= 3; n -= 2) h = __fma_rn(-(double)n * u, h, 1.0);
    const double q = __dmul_rn(-u, h);
    // 1 + p = exp(-d): p = -d (1 - d/2 (1 - d/3 (1 - d/4 (1 - d/5))))
    const double d = __dmul_rn(__dsub_rn(ax, z), __dadd_rn(ax, z));
    double t = __fma_rn(-d, 0.2, 1.0);
    t = __fma_rn(__dmul_rn(-d, 0.25), t, 1.0);
    t = __fma_rn(__ddiv_rn(-d, 3.0), t, 1.0);
    t = __fma_rn(__dmul_rn(-d, 0.5), t, 1.0);
    const double p = __dmul_rn(-d, t);
    const double g = __fma_rn(q, p, __dadd_rn(q, p));                 // (1 + q)(1 + p) - 1
    const double K_hi = 0x1.faf956cc3bebcp-1, K_lo = -0x1.b02ab54640020p-60;
    const double f_lo = __fma_rn(K_hi, g, K_lo);                      // F = K_hi + f_lo
    const double E = __dmul_rn(e1, 0x1p64);                           // exact
    const double ph = __dmul_rn(E, K_hi);
    const double pl = __fma_rn(E, K_hi, -ph);                         // E K_hi = ph + pl
    const double prod = __dmul_rn(__dadd_rn(ph, __fma_rn(E, f_lo, pl)), 0x1p-64);
    return __ddiv_rn(prod, ax);
}

__device__ __forceinline__ double erfc_tab(double x, const double* tbl) {
    const double ax = fabs(x);
    double r;
    if (ax < kErfcXMax) {
        const int k = __double2int_rn(ax * kErfcPerUnit);
        const double d = ax - (double)k * (1.0 / kErfcPerUnit);  // exact: k / 128
        const double* c = tbl + (size_t)k * kErfcTerms;
        r = c[kErfcTerms - 1];
#pragma unroll
        for (int n = kErfcTerms - 2; n >= 0; --n) r = fma(r, d, c[n]);
    } else {
        r = erfc_tail(ax);
    }
    return x < 0.0 ? 2.0 - r : r;
}

// 0.70710678118654752440 rounded to double, the reference's M_SQRT1_2
#define HPDEX_SQRT1_2 0.70710678118654752440

// ---------------------------------------------------------------------------------------
// Divisions by a known reciprocal. Markstein's theorem (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Develop. 34(1),
// 1990): if y is within half an ulp of 1/b and q within one ulp of a/b, then r = a - b q is
// exact in one fma and q + r y rounded once is a/b rounded to nearest (no overflow or
// underflow). So with y = RN(1/b) known in advance a correctly rounded quotient takes a
// multiply and two to four fmas instead of a full division. The results are the same doubles
// as IEEE division (__ddiv_rn); hpdex_selftest_division checks that on the device.
// ---------------------------------------------------------------------------------------
// a / b from y = RN(1/b). a * y rounded is within 1.5 ulp of a / b; one refinement brings the
// quotient within an ulp, and the second step rounds it correctly.
__device__ __forceinline__ double div_by_recip(double a, double b, double y) {
    const double q0 = __dmul_rn(a, y);
    const double q1 = __fma_rn(__fma_rn(-b, q0, a), y, q0);
    return __fma_rn(__fma_rn(-b, q1, a), y, q1);
}

// x / 12. RN(1/12) = (1 - 2^-54) / 12, so x * RN(1/12) rounded is within an ulp of x / 12 and
// a single step rounds it correctly.
__device__ __forceinline__ double div12(double x) {
    const double y = 0.083333333333333329;  // RN(1/12)
    const double q0 = __dmul_rn(x, y);
    return __fma_rn(__fma_rn(-12.0, q0, x), y, q0);
}

// Per-target constants of the asymptotic p-value when n1 and n2 do not depend on the gene
// (zero_handling min / max / mix), computed once on the host in the same rounded operations
// as p_asymptotic: N + 1, n1 n2, n1 n2 / 2, N (N - 1) and RN(1 / (N (N - 1))).
struct PConst {
    double N1, nm, mu, denom, rden;
};

inline PConst make_pconst(double n1, double n2) {
    PConst k;
    const double N = n1 + n2;
    k.N1 = N + 1.0;
    k.nm = n1 * n2;
    k.mu = 0.5 * k.nm;
    k.denom = N * (N - 1.0);
    k.rden = k.denom > 0.0 ? 1.0 / k.denom : 0.0;
    return k;
}

// p from the variance onwards (shared by both entry points below)
__device__ __forceinline__ double p_from_var(double U1, double nm, double mu, double var,
                                             double cc, int alt, const double* tbl) {
    const double sigma = (var > 0.0) ? __dsqrt_rn(var) : 0.0;
    double p = 1.0;
    if (alt == ALT_TWO_SIDED) {
        const double U2 = __dsub_rn(nm, U1);
        const double U = (U1 > U2 ? U1 : U2);
        if (sigma > 0.0) {
            const double z = __ddiv_rn(__dsub_rn(__dsub_rn(U, mu), cc), sigma);
            p = __dmul_rn(2.0, __dmul_rn(0.5, erfc_tab(__dmul_rn(z, HPDEX_SQRT1_2), tbl)));
            if (p > 1.0) p = 1.0;
            if (p < 0.0) p = 0.0;
        }
        return p;
    }
    const double U = (alt == ALT_LESS) ? __dsub_rn(nm, U1) : U1;
    if (sigma > 0.0) {
        const double z = __ddiv_rn(__dsub_rn(__dsub_rn(U, mu), cc), sigma);
        p = __dmul_rn(0.5, erfc_tab(__dmul_rn(z, HPDEX_SQRT1_2), tbl));
    }
    return (p < 0.0 ? 0.0 : (p > 1.0 ? 1.0 : p));
}

// n1, n2 per test (zero_handling none).
__device__ __forceinline__ double p_asymptotic(double U1, double n1, double n2, double tie_sum,
                                               double cc, int alt, const double* tbl) {
    const double N = __dadd_rn(n1, n2);
    const double nm = __dmul_rn(n1, n2);
    const double mu = __dmul_rn(0.5, nm);
    double tie_term = 0.0;
    const double denom = __dmul_rn(N, __dsub_rn(N, 1.0));
    if (denom > 0.0) tie_term = __ddiv_rn(tie_sum, denom);
    const double var = div12(__dmul_rn(nm, __dsub_rn(__dadd_rn(N, 1.0), tie_term)));
    return p_from_var(U1, nm, mu, var, cc, alt, tbl);
}

// Per-target constants (the same value as p_asymptotic with that target's n1, n2).
__device__ __forceinline__ double p_asymptotic_k(double U1, const PConst& k, double tie_sum,
                                                 double cc, int alt, const double* tbl) {
    double tie_term = 0.0;
    if (k.denom > 0.0) tie_term = div_by_recip(tie_sum, k.denom, k.rden);
    const double var = div12(__dmul_rn(k.nm, __dsub_rn(k.N1, tie_term)));
    return p_from_var(U1, k.nm, k.mu, var, cc, alt, tbl);
}

// fast_norm = true: the reference's scalar fast path (AI4Cell/hpdex src/cpp/include/
// common.hpp:14-92), restated: erfc from the Chebyshev fit erfcc of Numerical Recipes (Press et
// al., section 6.2; fractional error below 1.2e-7) with the math library's exp, mu and
// 1/sigma as precompute_mu_inv_sd computes them, z = (|U1 - mu| - cc) / sigma two-sided,
// (U1 - mu - cc) / sigma greater, (U1 - mu + cc) / sigma with p = 1 - sf less. (The
// reference's vectorised variant of the same polynomial nests its terms differently, so its
// values depend on the host's vector width; the scalar form is the one restated here.)
// Every operation is an explicitly rounded intrinsic in the C expression's order (as the
// oracle, compiled without contraction, evaluates it), so the value does not depend on the
// kernel the function is inlined into.
__device__ __forceinline__ double erfcc_nr(double x) {
    const double ax = fabs(x);
    const double t = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(0.5, ax)));
    double h = 0.17087277;
    h = __dadd_rn(-0.82215223, __dmul_rn(t, h));
    h = __dadd_rn(1.48851587, __dmul_rn(t, h));
    h = __dadd_rn(-1.13520398, __dmul_rn(t, h));
    h = __dadd_rn(0.27886807, __dmul_rn(t, h));
    h = __dadd_rn(-0.18628806, __dmul_rn(t, h));
    h = __dadd_rn(0.09678418, __dmul_rn(t, h));
    h = __dadd_rn(0.37409196, __dmul_rn(t, h));
    h = __dadd_rn(1.00002368, __dmul_rn(t, h));
    const double arg = __dadd_rn(__dsub_rn(__dmul_rn(-ax, ax), 1.26551223), __dmul_rn(t, h));
    const double tau = __dmul_rn(t, exp(arg));
    double r = (x >= 0.0) ? tau : __dsub_rn(2.0, tau);
    return r < 0.0 ? 0.0 : (r > 2.0 ? 2.0 : r);
}

__device__ __forceinline__ double p_asymptotic_fast(double U1, double n1, double n2,
                                                    double tie_sum, double cc, int alt) {
    const double N = __dadd_rn(n1, n2);
    const double nm = __dmul_rn(n1, n2);
    const double mu = __dmul_rn(__dmul_rn(0.5, n1), n2);
    const double denom = __dmul_rn(N, __dsub_rn(N, 1.0));
    const double var = (denom > 0.0)
        ? __dmul_rn(__ddiv_rn(nm, 12.0), __dsub_rn(__dadd_rn(N, 1.0), __ddiv_rn(tie_sum, denom)))
        : __ddiv_rn(__dmul_rn(nm, __dadd_rn(N, 1.0)), 12.0);
    const double inv_sd = (var <= 0.0) ? 0.0 : __ddiv_rn(1.0, __dsqrt_rn(var));
    if (inv_sd == 0.0) return 1.0;
    const double s2 = 1.4142135623730951;  // sqrt(2.0) rounded to double
    if (alt == ALT_TWO_SIDED)
        return __dmul_rn(2.0, __dmul_rn(0.5, erfcc_nr(__ddiv_rn(
            __dmul_rn(__dsub_rn(fabs(__dsub_rn(U1, mu)), cc), inv_sd), s2))));
    if (alt == ALT_GREATER)
        return __dmul_rn(0.5, erfcc_nr(__ddiv_rn(
            __dmul_rn(__dsub_rn(__dsub_rn(U1, mu), cc), inv_sd), s2)));
    return __dsub_rn(1.0, __dmul_rn(0.5, erfcc_nr(__ddiv_rn(
        __dmul_rn(__dadd_rn(__dsub_rn(U1, mu), cc), inv_sd), s2))));
}

}  // namespace hpdex
