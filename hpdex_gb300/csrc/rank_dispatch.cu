// rank_dispatch.cu -- dtype switch over the per-type rank kernel translation units.
#include "../../include/hpdex_gb300.h"
#include "rank_launch.h"

namespace hpdex {

cudaError_t rank_launch(int dtype, const RankArgs& a, int grid, size_t smem, cudaStream_t s) {
    switch (dtype) {
    case HPDEX_INT8: return rank_launch_i8(a, grid, smem, s);
    case HPDEX_UINT8: return rank_launch_u8(a, grid, smem, s);
    case HPDEX_INT16: return rank_launch_i16(a, grid, smem, s);
    case HPDEX_UINT16: return rank_launch_u16(a, grid, smem, s);
    case HPDEX_INT32: return rank_launch_i32(a, grid, smem, s);
    case HPDEX_UINT32: return rank_launch_u32(a, grid, smem, s);
    case HPDEX_INT64: return rank_launch_i64(a, grid, smem, s);
    case HPDEX_UINT64: return rank_launch_u64(a, grid, smem, s);
    case HPDEX_FLOAT32: return rank_launch_f32(a, grid, smem, s);
    case HPDEX_FLOAT64: return rank_launch_f64(a, grid, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t rank_occupancy(int dtype, size_t smem, size_t smem_optin, int acc_in_smem,
                           int* blocks) {
    switch (dtype) {
    case HPDEX_INT8: return rank_occupancy_i8(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_UINT8: return rank_occupancy_u8(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_INT16: return rank_occupancy_i16(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_UINT16: return rank_occupancy_u16(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_INT32: return rank_occupancy_i32(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_UINT32: return rank_occupancy_u32(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_INT64: return rank_occupancy_i64(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_UINT64: return rank_occupancy_u64(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_FLOAT32: return rank_occupancy_f32(smem, smem_optin, acc_in_smem, blocks);
    case HPDEX_FLOAT64: return rank_occupancy_f64(smem, smem_optin, acc_in_smem, blocks);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace hpdex
