// rank_i16.cu -- rank kernel instantiations for int16_t values.
#define HPDEX_RANK_T i16
#define HPDEX_RANK_V int16_t
#include "rank_impl.cuh"
