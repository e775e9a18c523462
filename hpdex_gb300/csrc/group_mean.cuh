// group_mean.cuh -- per (gene, group) means over a CSC matrix (sm_103a).
//
// Restates hpdex::group_mean_core (AI4Cell/hpdex src/cpp/mannwhitneyu.cpp:1118-1192): for
// every gene and group, the sum of the finite explicit values of rows in the group divided
// by group_rows[g] - invalid[g] (include_zeros; implicit zeros count, non-finite entries
// do not) or by valid[g] (explicit values only); a zero denominator gives 0. Output is
// flat [gene * G + g] like the reference. One CTA per gene; the per-group sums are double
// shared-memory atomics (any order; for float32 data whose per-gene magnitudes span less
// than ~2^29 the double sum of a few thousand values is exact, so the order is immaterial).
#pragma once
#include <cstdint>

#include "common.cuh"

namespace hpdex {

struct MeanArgs {
    const void* data;
    const int32_t* rows;
    const int64_t* indptr;
    int64_t n_rows;
    int32_t n_cols;
    int32_t G;
    const int32_t* gid;
    const long long* group_rows;
    int32_t include_zeros;
    double* out;                   // [n_cols * G]
    unsigned char* acc_global;     // per CTA 16*G bytes when not in shared memory
    int32_t acc_in_smem;
};

template <class V, int NT>
__global__ void __launch_bounds__(NT) group_mean_kernel(const MeanArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int G = a.G, tid = threadIdx.x;
    unsigned char* base = a.acc_in_smem ? smem : a.acc_global + (size_t)blockIdx.x * 16 * G;
    double* sum = reinterpret_cast<double*>(base);
    uint32_t* valid = reinterpret_cast<uint32_t*>(sum + G);
    uint32_t* invalid = valid + G;
    const V* data = reinterpret_cast<const V*>(a.data);

    for (int c = blockIdx.x; c < a.n_cols; c += gridDim.x) {
        for (int g = tid; g < G; g += NT) { sum[g] = 0.0; valid[g] = 0u; invalid[g] = 0u; }
        __syncthreads();
        const long long p0 = a.indptr[c], p1 = a.indptr[c + 1];
        for (long long p = p0 + tid; p < p1; p += NT) {
            const long long r = a.rows[p];
            if (r < 0 || r >= a.n_rows) continue;
            const int g = a.gid[r];
            if (g < 0 || g >= G) continue;
            const V v = data[p];
            if (Val<V>::finite(v)) {
                atomicAdd(&sum[g], Val<V>::to_double(v));
                atomicAdd(&valid[g], 1u);
            } else {
                atomicAdd(&invalid[g], 1u);
            }
        }
        __syncthreads();
        for (int g = tid; g < G; g += NT) {
            const long long denom = a.include_zeros ? (a.group_rows[g] - (long long)invalid[g])
                                                    : (long long)valid[g];
            a.out[(size_t)c * G + g] = denom > 0 ? __ddiv_rn(sum[g], (double)denom) : 0.0;
        }
        __syncthreads();
    }
}

}  // namespace hpdex
