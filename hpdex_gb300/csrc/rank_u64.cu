// rank_u64.cu -- rank kernel instantiations for uint64_t values.
#define HPDEX_RANK_T u64
#define HPDEX_RANK_V uint64_t
#include "rank_impl.cuh"
