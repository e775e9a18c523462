// rank_i32.cu -- rank kernel instantiations for int32_t values.
#define HPDEX_RANK_T i32
#define HPDEX_RANK_V int32_t
#include "rank_impl.cuh"
