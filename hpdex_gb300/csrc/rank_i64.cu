// rank_i64.cu -- rank kernel instantiations for int64_t values.
#define HPDEX_RANK_T i64
#define HPDEX_RANK_V int64_t
#include "rank_impl.cuh"
