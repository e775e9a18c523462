// Stand-in for the reference's third-party include bundle, used only to build the
// reference's own CPU kernel here for the oracle tests. The reference pulls OpenMP and
// Google Highway (an un-vendored, unpinned submodule that is empty in this checkout).
// Only VQSortStatic(ptr, n, SortAscending()) is reached on the precise path
// (src/cpp/mannwhitneyu.cpp:882); an exact std::sort gives the same sorted order,
// so U1 / tie sums / precise p-values are unchanged -- only CPU speed differs.
#pragma once
#include "config.hpp"
#include <omp.h>
#include <algorithm>
#include <cstddef>

namespace hwy {
struct SortAscending {};
namespace HWY_NAMESPACE {
template <class T>
inline void VQSortStatic(T* p, size_t n, SortAscending) { std::sort(p, p + n); }
}  // namespace HWY_NAMESPACE
}  // namespace hwy
