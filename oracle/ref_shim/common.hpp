// Stand-in for the reference's fast_norm p-value kernels (src/cpp/include/common.hpp),
// which need Highway's vector exp. The oracle build only supports fast_norm=False:
// the fast entry points raise instead of returning numbers that were never pinned.
#pragma once
#include "macro.hpp"
#include "simd.hpp"
#include <cstddef>
#include <stdexcept>

namespace hpdex {
inline void array_p_asymptotic_two_sided(const double*, const double*, const double*,
                                         const double*, const double*, double*, size_t) {
    throw std::runtime_error("fast_norm is unavailable in the oracle build of the reference");
}
inline void array_p_asymptotic_greater(const double*, const double*, const double*,
                                       const double*, const double*, double*, size_t) {
    throw std::runtime_error("fast_norm is unavailable in the oracle build of the reference");
}
inline void array_p_asymptotic_less(const double*, const double*, const double*,
                                    const double*, const double*, double*, size_t) {
    throw std::runtime_error("fast_norm is unavailable in the oracle build of the reference");
}
}  // namespace hpdex
