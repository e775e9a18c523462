// rank_launch.h -- host entry points of the rank kernel, one translation unit per value
// type (rank_<type>.cu) so that the instantiations compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include "mwu_rank.cuh"

namespace hpdex {
// Launches mwu_rank_kernel<V> for the dtype code `dtype` (HPDEX_* codes).
cudaError_t rank_launch(int dtype, const RankArgs& a, int grid, size_t smem, cudaStream_t s);
// Raises the kernel's dynamic shared-memory limit to the device maximum and reports how
// many CTAs of `smem` bytes fit on an SM.
cudaError_t rank_occupancy(int dtype, size_t smem, size_t smem_optin, int acc_in_smem,
                           int* blocks);
// per-type implementations
#define HPDEX_RANK_DECL(T)                                                                    \
    cudaError_t rank_launch_##T(const RankArgs& a, int grid, size_t smem, cudaStream_t s);   \
    cudaError_t rank_occupancy_##T(size_t smem, size_t smem_optin, int acc_in_smem, int* blocks);
HPDEX_RANK_DECL(i8)
HPDEX_RANK_DECL(u8)
HPDEX_RANK_DECL(i16)
HPDEX_RANK_DECL(u16)
HPDEX_RANK_DECL(i32)
HPDEX_RANK_DECL(u32)
HPDEX_RANK_DECL(i64)
HPDEX_RANK_DECL(u64)
HPDEX_RANK_DECL(f32)
HPDEX_RANK_DECL(f64)
#undef HPDEX_RANK_DECL
}  // namespace hpdex
