/* acceles_baseline.h -- library-SpMV comparison arm (libaes_baseline.so), for timing only.
 *
 * The reference's GPU baselines score every row with a library SpMV and sort all scores
 * (src/gpu/host_spmv_topk_csr_gpu_int8.cu: cusparseSpMV, thrust::sort_by_key, get_topk;
 * SpMV :68-314).  This is that method on GB300 over the FP32 CSR: cuSPARSE SpMV, a full
 * descending radix sort of the row scores, the first K.  It has no low-bit stage; equal scores
 * come out in ascending row order.  Kept out of libacceles.so so the engine does not load
 * cuSPARSE. */
#ifndef ACCELES_BASELINE_H
#define ACCELES_BASELINE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Upload the CSR (sorted; nnz < 2^31), then for each of nq host queries [nq][cols]: copy it
 * in, SpMV, sort all rows by score, copy the first k rows and scores out.  *ms_per_query is the
 * device time of SpMV + sort per query (events around them), averaged over all queries but the
 * first.  Returns the status codes of acceles.h. */
int aes_baseline_cusparse_topk(const uint64_t* ptr, const uint32_t* col, const float* val,
                               uint32_t rows, uint32_t cols, const float* queries, uint32_t nq,
                               uint32_t k, int device, uint32_t* out_idx, float* out_score,
                               double* ms_per_query);
const char* aes_baseline_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
