// rank_u32.cu -- rank kernel instantiations for uint32_t values.
#define HPDEX_RANK_T u32
#define HPDEX_RANK_V uint32_t
#include "rank_impl.cuh"
