// Stand-in for the reference's Highway SIMD helpers (src/cpp/include/simd.hpp).
// Nothing on the reference's MWU / group_mean path calls them; this header only
// satisfies the include, keeps the standard headers the original pulls in
// (<cstddef>, <utility>, <limits>, <cstring>) and supplies the OpenMP + sort shim.
#pragma once
#include <cstddef>
#include <cstring>
#include <limits>
#include <utility>
#include "dependencies.hpp"
