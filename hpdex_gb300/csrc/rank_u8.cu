// rank_u8.cu -- rank kernel instantiations for uint8_t values.
#define HPDEX_RANK_T u8
#define HPDEX_RANK_V uint8_t
#include "rank_impl.cuh"
