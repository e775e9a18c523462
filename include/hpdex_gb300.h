/*
 * hpdex_gb300.h -- C ABI of the GB300 (sm_103a) Mann-Whitney U differential-expression
 * backend. Plain pointers and sizes only; every entry point returns an int status
 * (HPDEX_OK = 0) and leaves a message for hpdex_last_error() on failure.
 *
 * Reference interfaces replaced (AI4Cell/hpdex):
 *   hpdex_mannwhitneyu  <- kernel.mannwhitneyu   src/cpp/module.cpp:196-228
 *                          hpdex::mannwhitneyu<T> src/cpp/mannwhitneyu.cpp:1067-1111
 *   hpdex_group_mean    <- kernel.group_mean      src/cpp/module.cpp:230-242
 *                          hpdex::group_mean<T>  src/cpp/mannwhitneyu.cpp:1275-1304
 *   hpdex_mwu_options   <- MannWhitneyuOption    src/cpp/include/mannwhitneyu.hpp:16-32
 *   the matrix arguments <- view::CscView<T>     src/cpp/include/sparse.hpp:41-68
 * The resident-matrix / plan / server entry points have no single counterpart: they split
 * the reference call into upload, launch and download so that matrices stay in HBM.
 *
 * Matrix: CSC, n_rows cells x n_cols genes; data[nnz] of `dtype`, indices[nnz] int64 row
 * ids, indptr[n_cols+1] int64. group_id[n_rows] int32: 0 = reference, 1..n_targets =
 * targets, anything else ignored. All host pointers unless stated otherwise.
 *
 * Output layout: U1_out and P_out are n_targets x n_cols row-major (target-major), i.e.
 * out[(g-1) * n_cols + gene]. The reference returns the transposed, gene-major order
 * (mannwhitneyu.cpp:959): reference_flat.reshape(n_cols, n_targets).T equals ours.
 */
#ifndef HPDEX_GB300_H
#define HPDEX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HPDEX_OK 0
#define HPDEX_ERR_RUNTIME 1  /* reference-style runtime_error (message text matches)  */
#define HPDEX_ERR_ARGUMENT 2 /* malformed input (sizes, pointers, indptr)              */
#define HPDEX_ERR_CUDA 3     /* CUDA runtime failure or no usable device               */
#define HPDEX_ERR_UNSUPPORTED 4
#define HPDEX_ERR_TIMEOUT 5  /* hpdex_server_wait: the query did not finish in time      */

/* dtype codes of `data` (the reference's TYPE_DISPATCH list, macro.hpp:4-14) */
#define HPDEX_INT8 0
#define HPDEX_UINT8 1
#define HPDEX_INT16 2
#define HPDEX_UINT16 3
#define HPDEX_INT32 4
#define HPDEX_UINT32 5
#define HPDEX_INT64 6
#define HPDEX_UINT64 7
#define HPDEX_FLOAT32 8
#define HPDEX_FLOAT64 9

/* zero_handling / alternative / method: the reference's enum values */
#define HPDEX_ZERO_NONE 0
#define HPDEX_ZERO_MIN 1
#define HPDEX_ZERO_MAX 2
#define HPDEX_ZERO_MIX 3
#define HPDEX_LESS 0
#define HPDEX_GREATER 1
#define HPDEX_TWO_SIDED 2
#define HPDEX_EXACT 1
#define HPDEX_ASYMPTOTIC 2

/* exact_variant: 0 = the reference's own exact p (mannwhitneyu.cpp:98-188, a bounded-
 * composition count in wrapping uint64), 1 = the true MWU null distribution (what
 * scipy.stats.mannwhitneyu(method="exact") computes). */
#define HPDEX_EXACT_REFERENCE 0
#define HPDEX_EXACT_MWU_NULL 1

typedef struct hpdex_mwu_options {
    int32_t ref_sorted;     /* accepted; sorting is never skipped, results are the same */
    int32_t tar_sorted;     /* accepted; see ref_sorted                                 */
    int32_t tie_correction; /* 1: use sum(t^3 - t) in the variance                      */
    int32_t use_continuity; /* 1: continuity correction 0.5                             */
    int32_t fast_norm;      /* 1: the reference's fast normal tail (NR erfcc)           */
    int32_t zero_handling;  /* HPDEX_ZERO_*                                             */
    int32_t alternative;    /* HPDEX_LESS / GREATER / TWO_SIDED                         */
    int32_t method;         /* HPDEX_EXACT / HPDEX_ASYMPTOTIC                           */
    int32_t exact_variant;  /* HPDEX_EXACT_REFERENCE / HPDEX_EXACT_MWU_NULL             */
} hpdex_mwu_options;

/* Fills `o` with the reference binding's defaults (module.cpp:215-227) except
 * fast_norm = 0. */
void hpdex_mwu_options_default(hpdex_mwu_options* o);

/* Message of the last failure on the calling thread ("" if none). */
const char* hpdex_last_error(void);

/* Number of visible CUDA devices (0 when none); never fails. */
int hpdex_device_count(void);

/* Streaming multiprocessors of the current device (152 on a GB300). */
int hpdex_device_sm_count(int32_t* sms);

/* Device memory of destroyed matrices, plans and finished one-shot calls stays cached for
 * reuse by later calls (no cudaMalloc/cudaFree per call); this returns it to the driver. */
int hpdex_release_cached_memory(void);

/* Page-locked host buffers for result arrays (the Python wrapper uses them for U1 / P): the
 * one-shot call writes results into such buffers directly, with no host pages to fault in.
 * acquire sets *ptr to a buffer of at least `bytes` bytes, or to NULL when the pool (2 GiB
 * held at most) cannot lend one: use ordinary memory then. release returns a buffer to the
 * pool; hpdex_release_cached_memory frees the idle ones. */
int hpdex_host_buffer_acquire(int64_t bytes, void** ptr);
int hpdex_host_buffer_release(void* ptr);

/* ---- DE post-processing on the device (the reference DE driver does these on the host,
 * de.py:138-142 and :174-184) ----
 * hpdex_bh_fdr: Benjamini-Hochberg adjusted p-values of p[0..n), as
 * scipy.stats.false_discovery_control(p, method="bh") (values outside [0, 1] or NaN:
 * HPDEX_ERR_ARGUMENT with scipy's message). hpdex_fold_change: from per-(gene, group) means
 * (gene-major [gene * n_groups + g], g = 0 the reference) the fold change and log2 fold
 * change per (target, gene), target-major: tar / ref, `clip` where ref < 1e-10, 1 / clip
 * where tar < 1e-10. Host pointers in and out. */
int hpdex_bh_fdr(const double* p, int64_t n, double* fdr);
int hpdex_fold_change(const double* means, int64_t n_genes, int64_t n_groups, double clip,
                      double* fold, double* log2fold);

/* Self-check of the p-value stage's table-based erfc against the CUDA math library's erfc
 * on n_points points spread over [-8, 27]: the largest relative difference (where erfc >=
 * 1e-300) and the largest absolute difference. */
int hpdex_selftest_erfc(int64_t n_points, double* max_rel_err, double* max_abs_err);

/* The p-value stage's erfc (table steps below 26.5, the deep-tail steps above) at n host
 * points x, into host out: lets a test compare it with the host C library's erfc, which the
 * reference calls (mannwhitneyu.cpp:21), including the subnormal tail. */
int hpdex_selftest_erfc_values(const double* x, int64_t n, double* out);

/* Self-check of the p-value stage's divisions by a precomputed reciprocal (Markstein's
 * correction steps) against IEEE division, bit for bit, on n_cases generated quotients (tie
 * sums over N (N - 1), random doubles, quotients next to a rounding midpoint, x / 12):
 * *mismatches = the number that differ (0 expected). */
int hpdex_selftest_division(int64_t n_cases, uint64_t seed, int64_t* mismatches);

/* ---- one-shot calls (reference semantics; host pointers in and out) ---- */

/* kernel.mannwhitneyu. threads is accepted for signature parity and only affects host-side
 * preparation. U1_out / P_out: n_targets * n_cols doubles, target-major. */
int hpdex_mannwhitneyu(int32_t dtype, const void* data, const int64_t* indices,
                       const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                       const int32_t* group_id, int64_t n_targets,
                       const hpdex_mwu_options* opt, int32_t threads, double* U1_out,
                       double* P_out);

/* hpdex_mannwhitneyu with int32 row ids (scipy's index type below 2^31 entries): the same
 * results, half the row-id bytes to upload, no cast to int64 on the host. */
int hpdex_mannwhitneyu_idx32(int32_t dtype, const void* data, const int32_t* indices,
                             const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                             const int32_t* group_id, int64_t n_targets,
                             const hpdex_mwu_options* opt, int32_t threads, double* U1_out,
                             double* P_out);

/* kernel.group_mean. out: n_cols * n_groups doubles, flat [gene * n_groups + g] exactly as
 * the reference. use_kahan is honoured as documented (the reference binding forwards
 * `threads` into it, module.cpp:211-213); both summation modes agree to ~1e-15 here. */
int hpdex_group_mean(int32_t dtype, const void* data, const int64_t* indices,
                     const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                     const int32_t* group_id, int64_t n_groups, int32_t include_zeros,
                     int32_t use_kahan, int32_t threads, double* out);

/* ---- resident matrices and plans (matrix stays in HBM across calls) ---- */

typedef struct hpdex_matrix hpdex_matrix;
typedef struct hpdex_plan hpdex_plan;

/* Uploads a CSC matrix to the current device in the library's resident layout
 * (values as given, row ids narrowed to int32 when n_rows < 2^31). */
int hpdex_matrix_create(int32_t dtype, const void* data, const int64_t* indices,
                        const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                        hpdex_matrix** out);
/* hpdex_matrix_create with int32 row ids, copied as they are (ids outside [0, n_rows) are
 * skipped by every kernel, as the int64 path's narrowing marks them). */
int hpdex_matrix_create_idx32(int32_t dtype, const void* data, const int32_t* indices,
                              const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                              hpdex_matrix** out);
/* The same resident matrix from a cells x genes CSR (AnnData's native layout; indptr over
 * the n_rows cells, indices = gene ids in [0, n_cols)), transposed on the device: columns hold
 * their rows in ascending order, entries with a gene id outside [0, n_cols) are dropped. */
int hpdex_matrix_create_csr(int32_t dtype, const void* data, const int64_t* indices,
                            const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                            hpdex_matrix** out);
/* hpdex_matrix_create_csr with int32 gene ids (scipy's index type), uploaded as they are. */
int hpdex_matrix_create_csr_idx32(int32_t dtype, const void* data, const int32_t* indices,
                                  const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                                  hpdex_matrix** out);
/* Per (gene, group) means of a resident matrix, flat [gene * n_groups + g]: the values of
 * hpdex_group_mean (reference group_mean_core, include_zeros as there). */
int hpdex_matrix_group_mean(const hpdex_matrix* m, const int32_t* group_id, int64_t n_groups,
                            int32_t include_zeros, double* out);
/* A resident matrix from data already on the device: values (dtype) and int32 row ids are
 * device pointers (copied into the library's own buffers; the caller keeps ownership), the
 * n_cols + 1 column pointers are host memory. Otherwise as hpdex_matrix_create_idx32. */
int hpdex_matrix_create_device(int32_t dtype, const void* d_data, const int32_t* d_rows,
                               const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                               hpdex_matrix** out);
int hpdex_matrix_destroy(hpdex_matrix* m);
int hpdex_matrix_info(const hpdex_matrix* m, int64_t* n_rows, int64_t* n_cols, int64_t* nnz,
                      int64_t* device_bytes);

/* A grouping over a resident matrix: validates it like the reference (errors raised before
 * any launch), uploads group_id, orders genes for the work queue and reserves outputs. */
int hpdex_plan_create(hpdex_matrix* m, const int32_t* group_id, int64_t n_targets,
                      const hpdex_mwu_options* opt, hpdex_plan** out);
int hpdex_plan_destroy(hpdex_plan* p);

/* Runs the MWU on the device. mode 0 = batched (persistent work-queue kernel, captured
 * in a CUDA graph), mode 1 = plain (one launch per gene, no graph, no queue). Results stay
 * on the device until hpdex_plan_download. Synchronous. */
#define HPDEX_MODE_BATCHED 0
#define HPDEX_MODE_PLAIN 1
int hpdex_plan_run(hpdex_plan* p, int32_t mode);

/* Asymptotic plans compute their p-values inside the rank kernel (on = 1, the default):
 * each gene's tests are finished by a few warps during the next gene's rank phase, so the
 * FP64 work overlaps the integer work. on = 0 runs a separate p-value kernel after the rank
 * kernel instead; the results are the same. Exact plans accept only on = 0. */
int hpdex_plan_set_fused_pvalues(hpdex_plan* p, int32_t on);

/* Copies U1 / P (n_targets x n_cols, target-major) to host; either pointer may be NULL. */
int hpdex_plan_download(hpdex_plan* p, double* U1_out, double* P_out);

/* Diagnostic: the rank kernel's bucket table of 2^bits entries (9..13; 13, the default, was
 * the fastest on every workload measured). A smaller table leaves more shared memory for a
 * gene's elements at the cost of larger buckets. The results do not depend on it. */
int hpdex_plan_set_bucket_bits(hpdex_plan* p, int32_t bits);

/* Diagnostic. Where the rank kernel keeps its per-warp run counters (16 bits per group):
 * mode 1 in shared memory (when the accumulators are there), 0 in global memory (its rounds
 * then resolve repeated groups by warp match, and the shared memory goes to elements), -1 (the
 * default) in shared memory up to 1,024 groups. The results are the same in every mode. */
int hpdex_plan_set_run_counters(hpdex_plan* p, int32_t mode);

/* Measures the plan under each candidate layout of the rank kernel -- run counters in shared
 * (1) or global (0) memory, bucket table of 2^13 or 2^12 entries -- as the mean CUDA-event time
 * of `reps` batched runs after one untimed run, and keeps the fastest. All candidates give the
 * same results. Outputs (each may be NULL): the chosen run-counter mode and bucket bits, and
 * the four mean times in ms in the order (1, 13), (1, 12), (0, 13), (0, 12). */
int hpdex_plan_autotune(hpdex_plan* p, int32_t reps, int32_t* run_counters_out,
                        int32_t* bucket_bits_out, float* ms_out);

/* The rank kernel takes each gene whose stored values are integers of magnitude below 2^31
 * (UMI counts) and whose value span times the number of groups fits its shared memory through
 * a histogram path: one counter per (value, group), rank sums from a prefix scan of the
 * reference's counts. on = 0 sends every gene through the general (bucket) path instead, on = 1
 * (the default) restores the per-gene choice. Both give the same results. */
int hpdex_plan_set_histogram(hpdex_plan* p, int32_t on);

/* Diagnostic. The rank kernel lets a warp resolve a large bucket while other warps of its CTA
 * are still listing them. By default (on = 0) a warp that finds the next list entry not yet
 * published leaves it to a pass after the next block barrier; on = 1 makes it wait for the entry
 * a bounded number of polls first (slower on the measured workloads). The results are the same
 * either way. */
int hpdex_plan_set_drain_wait(hpdex_plan* p, int32_t on);

/* Device times (ms, CUDA events on the launching stream) of the last hpdex_plan_run:
 * [0] whole run, [1] rank kernel(s) (with the p-values when fused), [2] p-value kernel
 * (0 when fused); and the number of kernel launches it made. */
int hpdex_plan_timings(const hpdex_plan* p, float* ms3, int32_t* launches);

/* ---- no-allocation variant (no counterpart in the reference) ----
 *
 * hpdex_mannwhitneyu_noalloc computes the same U1 / P as hpdex_mannwhitneyu but allocates
 * nothing: no cudaMalloc, no cudaFree, no allocating library routine. It is meant for
 * callers that cannot allocate device memory during a call -- code running inside a
 * framework's own memory pool or caching allocator (a raw cudaMalloc/cudaFree would bypass
 * the pool and can synchronise the device), serving loops that reserve all memory up front
 * for predictable latency, and plugin hosts that forbid allocation.
 *
 * The caller passes device pointers: d_data (the values in CSC order, d_indptr[n_cols] of
 * them), d_rows (int32 row ids, the library's resident layout), d_indptr (int64,
 * n_cols + 1), d_group_id (int32, n_rows) and the outputs d_U1 / d_P (n_targets * n_cols
 * doubles, target-major). `stream` is a cudaStream_t (NULL = legacy default stream). The call
 * synchronises that stream before returning.
 *
 * Working memory is one fixed device array of HPDEX_NOALLOC_SCRATCH_BYTES inside the
 * library; every GPU that loads the library holds it until the process exits. Limits:
 * n_targets + 1 <= HPDEX_NOALLOC_MAX_GROUPS, n_cols <= HPDEX_NOALLOC_MAX_COLS,
 * method = HPDEX_ASYMPTOTIC only, and the longest column must fit the per-SM element
 * slices that remain in the array (about 50k entries for float32 data with few rows and
 * targets). That column limit falls as n_rows and n_targets grow: the group ids take 2 bytes
 * per row of the array and the per-warp run counters up to about 15 MB at 1,024 groups, so
 * past roughly 30 million rows nothing is left. Anything beyond returns
 * HPDEX_ERR_UNSUPPORTED with a message that gives the limit computed for the call. Genes are
 * taken in column order (no longest-first scheduling).
 *
 * The first call on a device does a one-time set-up (it resolves the device address of
 * the array with cudaGetSymbolAddress). Every call shares the one array and finds the previous call's contents in it: calls
 * that overlap on the GPU (two host threads, or two streams) race and corrupt each other,
 * so serialise them.
 */
#define HPDEX_NOALLOC_SCRATCH_BYTES (64u << 20)
#define HPDEX_NOALLOC_MAX_GROUPS 1024
#define HPDEX_NOALLOC_MAX_COLS 262144
int hpdex_mannwhitneyu_noalloc(int32_t dtype, const void* d_data, const int32_t* d_rows,
                               const int64_t* d_indptr, int64_t n_rows, int64_t n_cols,
                               const int32_t* d_group_id, int64_t n_targets,
                               const hpdex_mwu_options* opt, double* d_U1, double* d_P,
                               void* stream);

/* ---- serving loop (the reference has none; its DE driver runs one grouping per call) ----
 *
 * A server keeps resident matrices (hpdex_matrix handles, borrowed: keep them alive until
 * the server is destroyed) and answers DE queries -- a grouping and target count over one of
 * them -- as they arrive. A worker thread admits pending queries in arrival order while their
 * device workspace (outputs, group ids: about 16 B x n_targets x n_cols + 6 B x n_rows) fits
 * in `workspace_bytes`, coalesces up to `max_batch` admitted queries of one value dtype into
 * one launch of the persistent rank kernel (the (query, gene) work items share one
 * longest-first queue), then runs their p-value kernels and writes U1 and P into the
 * caller's arrays. The next batch is prepared and queued on the GPU while the previous one
 * runs. max_batch = 1 gives per-query launches. Asymptotic p-values only.
 *
 * hpdex_server_submit copies group_id; U1_out and P_out (n_targets x n_cols doubles,
 * target-major, host memory) must stay valid until hpdex_server_wait returns for that
 * query. hpdex_server_wait returns the query's status (HPDEX_OK, or the error the query
 * raised, with its message for hpdex_last_error), or HPDEX_ERR_TIMEOUT when it is still
 * running after timeout_s seconds (a negative timeout waits without limit); latency_ms (may
 * be NULL) is the time from submission to completion. A query is forgotten once waited for.
 */
typedef struct hpdex_server hpdex_server;
int hpdex_server_create(int64_t workspace_bytes, int32_t max_batch, hpdex_server** out);
int hpdex_server_add_matrix(hpdex_server* s, hpdex_matrix* m, int32_t* matrix_id);
int hpdex_server_submit(hpdex_server* s, int32_t matrix_id, const int32_t* group_id,
                        int64_t n_targets, const hpdex_mwu_options* opt, double* U1_out,
                        double* P_out, int64_t* query_id);
int hpdex_server_wait(hpdex_server* s, int64_t query_id, double timeout_s, double* latency_ms);
/* completed queries, launches (batches) and summed GPU busy time (ms) since creation */
int hpdex_server_stats(const hpdex_server* s, int64_t* completed, int64_t* batches,
                       double* busy_ms);
/* Where a server's time went, summed over its batches: host time preparing and queueing them
 * (prep_ms: group-id copies, task tables, launches), device time of the rank launches and of
 * the p-value launches (one per batch), in ms. */
int hpdex_server_phase_stats(const hpdex_server* s, double* prep_ms, double* rank_ms, double* pvalue_ms);
/* finishes the admitted work, fails queries still pending, joins the worker */
int hpdex_server_destroy(hpdex_server* s);

#ifdef __cplusplus
}
#endif
#endif /* HPDEX_GB300_H */
