// rank_impl.cuh -- body of one per-type translation unit of the rank kernel; the including
// file defines HPDEX_RANK_T (suffix) and HPDEX_RANK_V (value type).
#include "rank_launch.h"

namespace hpdex {

#define HPDEX_CAT2(a, b) a##b
#define HPDEX_CAT(a, b) HPDEX_CAT2(a, b)

cudaError_t HPDEX_CAT(rank_launch_, HPDEX_RANK_T)(const RankArgs& a, int grid, size_t smem,
                                                  cudaStream_t s) {
    // (accumulators in shared memory, histogram path, decoded-copy compaction, run counters in
    // global memory)
    auto k = !a.acc_in_smem   ? mwu_rank_kernel<HPDEX_RANK_V, 1024, false, false, true, false>
             : !a.cnt_in_smem  ? mwu_rank_kernel<HPDEX_RANK_V, 1024, true, false, true, true>
             : !a.no_histogram ? mwu_rank_kernel<HPDEX_RANK_V, 1024, true, true, true, false>
             : a.any_compact   ? mwu_rank_kernel<HPDEX_RANK_V, 1024, true, false, true, false>
                               : mwu_rank_kernel<HPDEX_RANK_V, 1024, true, false, false, false>;
    k<<<grid, 1024, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t HPDEX_CAT(rank_occupancy_, HPDEX_RANK_T)(size_t smem, size_t smem_optin,
                                                     int acc_in_smem, int* blocks) {
    // the variants of an accumulator layout get the same shared-memory limit
    decltype(&mwu_rank_kernel<HPDEX_RANK_V, 1024, true, true, true, false>) ks[4] = {
        acc_in_smem ? mwu_rank_kernel<HPDEX_RANK_V, 1024, true, false, false, false>
                    : mwu_rank_kernel<HPDEX_RANK_V, 1024, false, false, true, false>,
        acc_in_smem ? mwu_rank_kernel<HPDEX_RANK_V, 1024, true, false, true, false>
                    : mwu_rank_kernel<HPDEX_RANK_V, 1024, false, false, true, false>,
        acc_in_smem ? mwu_rank_kernel<HPDEX_RANK_V, 1024, true, true, true, false>
                    : mwu_rank_kernel<HPDEX_RANK_V, 1024, false, false, true, false>,
        acc_in_smem ? mwu_rank_kernel<HPDEX_RANK_V, 1024, true, false, true, true>
                    : mwu_rank_kernel<HPDEX_RANK_V, 1024, false, false, true, false>};
    for (auto k : ks) {
        cudaFuncAttributes fa;
        cudaError_t e = cudaFuncGetAttributes(&fa, k);
        if (e != cudaSuccess) return e;
        // the opt-in limit covers static + dynamic shared memory
        const int max_dyn = (int)(smem_optin - fa.sharedSizeBytes);
        if ((size_t)max_dyn < smem) return cudaErrorInvalidValue;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, ks[0], 1024, smem);
}

}  // namespace hpdex
