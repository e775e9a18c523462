/* One call of the reference's kernel.mannwhitneyu through the C ABI, from host arrays:
 * float32 CSC values, int64 row ids and column pointers, int32 group ids (0 reference,
 * 1..T targets, -1 ignored). U1 and P come back target-major, T x C doubles. */
#include <stdio.h>
#include <stdlib.h>

#include "hpdex_gb300.h"

int run_mwu(const float* data, const int64_t* indices, const int64_t* indptr, int64_t n_rows,
            int64_t n_cols, int64_t nnz, const int32_t* group_id, int64_t T) {
    hpdex_mwu_options o;
    hpdex_mwu_options_default(&o);
    o.zero_handling = HPDEX_ZERO_MIN;
    o.use_continuity = 1;
    const int64_t C = n_cols;
    double* U1 = malloc((size_t)(T * C) * sizeof(double));
    double* P = malloc((size_t)(T * C) * sizeof(double));
    int st = hpdex_mannwhitneyu(HPDEX_FLOAT32, data, indices, indptr, n_rows, n_cols, nnz,
                                group_id, T, &o, -1, U1, P);
    if (st != HPDEX_OK) fprintf(stderr, "%s\n", hpdex_last_error());
    free(U1);
    free(P);
    return st;
}
