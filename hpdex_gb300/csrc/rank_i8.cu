// rank_i8.cu -- rank kernel instantiations for int8_t values.
#define HPDEX_RANK_T i8
#define HPDEX_RANK_V int8_t
#include "rank_impl.cuh"
