// Harness around the reference's own scalar fast normal tail (AI4Cell/hpdex
// src/cpp/include/common.hpp: fast_erfc, normal_sf, precompute_mu_inv_sd and the three
// p_asymptotic_* functions, the lines before its SIMD section). oracle/build_ref.sh copies
// that block, unmodified, into oracle/_ref/ref_fast_scalar_block.hpp at build time and
// compiles this file against it; nothing of the reference is kept in the repository.
//
// TEST INFRASTRUCTURE ONLY: tests/ load the resulting oracle/_ref/libref_fast_scalar.so to pin
// the oracle's restatement of the fast_norm p-values (oracle_p_asymptotic_fast) to the
// reference's code. The block needs only <cmath> and the reference's force_inline_ macro.
#include <cmath>
#include <cstddef>
#include <cstdint>

#define force_inline_ inline

namespace hpdex {
#include "ref_fast_scalar_block.hpp"
}  // namespace hpdex

// p for arrays of tests, as the reference's scalar functions compute it; alternative:
// 0 less, 1 greater, 2 two-sided (the reference's enum).
extern "C" void ref_fast_p(const double* U1, const double* n1, const double* n2,
                           const double* tie_sum, double cc, int alternative, int64_t n,
                           double* out) {
    for (int64_t i = 0; i < n; ++i) {
        double mu = 0.0, inv_sd = 0.0;
        const size_t a = static_cast<size_t>(n1[i]), b = static_cast<size_t>(n2[i]);
        if (alternative == 2)
            out[i] = hpdex::p_asymptotic_two_sided(U1[i], a, b, tie_sum[i], cc, mu, inv_sd);
        else if (alternative == 1)
            out[i] = hpdex::p_asymptotic_greater(U1[i], a, b, tie_sum[i], cc, mu, inv_sd);
        else
            out[i] = hpdex::p_asymptotic_less(U1[i], a, b, tie_sum[i], cc, mu, inv_sd);
    }
}
