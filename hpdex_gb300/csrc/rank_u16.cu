// rank_u16.cu -- rank kernel instantiations for uint16_t values.
#define HPDEX_RANK_T u16
#define HPDEX_RANK_V uint16_t
#include "rank_impl.cuh"
