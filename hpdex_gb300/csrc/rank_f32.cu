// rank_f32.cu -- rank kernel instantiations for float values.
#define HPDEX_RANK_T f32
#define HPDEX_RANK_V float
#include "rank_impl.cuh"
