// transpose.cuh -- cells x genes CSR (AnnData's native layout) to the resident CSC layout
// on the device (sm_103a), so that the DE driver does not transpose on the host (the
// reference driver calls scipy's tocsc(), src/hpdex/de.py:106-107).
//
// Stable: within each output column the row ids ascend, as in a CSC built on the host.
//   1. per-block column counts: block b takes rows [b * rpb, (b + 1) * rpb); a shared-memory
//      histogram of its entries' gene ids goes to cnt[b][c]
//   2. per column, an exclusive scan over the blocks plus the column's start gives each block
//      its first output position in every column (and the column totals give the pointers)
//   3. scatter: block b walks its rows in order, one row per step, every entry taking the
//      next position of its column from a shared-memory cursor; the step ends with a block
//      barrier, so a later row always lands after an earlier one
// Entries with a gene id outside [0, n_genes) are dropped (the reference skips row ids
// outside the matrix the same way). Row ids come out as int32 (n_rows < 2^31).
#pragma once
#include <cstdint>

#include "common.cuh"

namespace hpdex {

constexpr int kTransposeThreads = 256;

// cnt[b * n_genes + c]: entries of rows [b*rpb, (b+1)*rpb) in column c. SMEM: a shared-memory
// histogram (n_genes fits); else atomics straight into the block's row of cnt (zeroed first).
template <bool SMEM, class GI>  // GI: gene id type (int32 or int64)
__global__ void __launch_bounds__(kTransposeThreads) csr_block_count_kernel(
    const int64_t* indptr, const GI* genes, long long n_rows, long long rpb, int n_genes,
    uint32_t* cnt) {
    extern __shared__ uint32_t hist_s[];
    uint32_t* out = cnt + (size_t)blockIdx.x * n_genes;
    uint32_t* hist = SMEM ? hist_s : out;
    if constexpr (SMEM) {
        for (int c = threadIdx.x; c < n_genes; c += kTransposeThreads) hist[c] = 0u;
        __syncthreads();
    }
    const long long r0 = (long long)blockIdx.x * rpb, r1 = min(n_rows, r0 + rpb);
    if (r0 < r1) {
        const long long e0 = indptr[r0], e1 = indptr[r1];
        for (long long e = e0 + threadIdx.x; e < e1; e += kTransposeThreads) {
            const int64_t g = genes[e];
            if (g >= 0 && g < n_genes) atomicAdd(&hist[g], 1u);
        }
    }
    if constexpr (SMEM) {
        __syncthreads();
        for (int c = threadIdx.x; c < n_genes; c += kTransposeThreads) out[c] = hist[c];
    }
}

// Per column c (one thread each): the column's total, and cnt[b][c] replaced by the block's
// offset inside the column (exclusive scan over blocks).
__global__ void csr_column_scan_kernel(uint32_t* cnt, int nblocks, int n_genes, int64_t* col_total) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_genes) return;
    uint32_t run = 0;
    for (int b = 0; b < nblocks; ++b) {
        uint32_t* p = cnt + (size_t)b * n_genes + c;
        const uint32_t v = *p;
        *p = run;
        run += v;
    }
    col_total[c] = run;
}

// Exclusive scan of col_total[0..n) into indptr[0..n] (one block of 1024 threads).
__global__ void __launch_bounds__(1024) column_pointer_scan_kernel(const int64_t* col_total, int n,
                                                                   int64_t* indptr) {
    __shared__ long long ws[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (n + 1023) / 1024;
    const int beg = min(n, tid * per), end = min(n, beg + per);
    long long s = 0;
    for (int i = beg; i < end; ++i) s += col_total[i];
    long long incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        const long long x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        long long v = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const long long x = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += x;
        }
        ws[lane] = v - ws[lane];  // exclusive over warps
    }
    __syncthreads();
    long long o = ws[warp] + incl - s;
    for (int i = beg; i < end; ++i) {
        indptr[i] = o;
        o += col_total[i];
    }
    if (tid == 1023) indptr[n] = o;
}

// SMEM: cursors in shared memory; else the block's row of offs serves as its cursors.
template <class V, bool SMEM, class GI>
__global__ void __launch_bounds__(kTransposeThreads) csr_scatter_kernel(
    const int64_t* indptr, const GI* genes, const V* vals, long long n_rows, long long rpb,
    int n_genes, uint32_t* offs, const int64_t* col_ptr, int32_t* rows_out, V* vals_out) {
    extern __shared__ uint32_t cursor_s[];
    uint32_t* o = offs + (size_t)blockIdx.x * n_genes;
    uint32_t* cursor = SMEM ? cursor_s : o;
    if constexpr (SMEM) {
        for (int c = threadIdx.x; c < n_genes; c += kTransposeThreads) cursor[c] = o[c];
        __syncthreads();
    }
    const long long r0 = (long long)blockIdx.x * rpb, r1 = min(n_rows, r0 + rpb);
    for (long long r = r0; r < r1; ++r) {
        const long long e0 = indptr[r], e1 = indptr[r + 1];
        for (long long e = e0 + threadIdx.x; e < e1; e += kTransposeThreads) {
            const int64_t g = genes[e];
            if (g >= 0 && g < n_genes) {
                const long long pos = col_ptr[g] + atomicAdd(&cursor[g], 1u);
                rows_out[pos] = (int32_t)r;
                vals_out[pos] = vals[e];
            }
        }
        __syncthreads();
    }
}

}  // namespace hpdex
