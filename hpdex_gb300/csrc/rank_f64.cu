// rank_f64.cu -- rank kernel instantiations for double values.
#define HPDEX_RANK_T f64
#define HPDEX_RANK_V double
#include "rank_impl.cuh"
