/*
 * ref_shim.cpp -- C entry points over the reference's own CPU gold code.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the reference headers where
 * they lie (include path given on the command line), into oracle/_ref/libaes_ref.so, which is
 * never committed.  Tests use it to pin the C restatement in aes_oracle.c; bench.py's reference
 * arm may time it when it exists for the running machine.  Nothing here is product code.
 *
 * Wrapped reference functions (zhaijiaqi/AccelES):
 *   spmv_coo_gold_top_k_2   src/fpga/src/gold_algorithms/gold_algorithms.hpp:249-308
 *   spmv_coo_gold_top_k     src/fpga/src/gold_algorithms/gold_algorithms.hpp:189-247
 *   spmv_coo_gold4          src/fpga/src/gold_algorithms/gold_algorithms.hpp:141-187
 *   sort_tuples / sort_pr   src/common/utils/evaluation_utils.hpp:16-62
 *   readMtx                 src/common/utils/utils.hpp:450-492 (with readTuples, undirect,
 *                           customSort :331-437 and mmio.hpp)
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

/* The reference headers rely on <cmath>/<cstring> being included before them. */
using std::log2;

#include "common/types.hpp"
#include "common/csc_matrix/csc_matrix.hpp"
#include "common/utils/evaluation_utils.hpp"
#include "common/utils/utils.hpp"
#include "fpga/src/gold_algorithms/gold_algorithms.hpp"

extern "C" {

void ref_gold_topk2_i32(const uint32_t* row, const uint32_t* col, const int32_t* val, uint64_t nnz,
                        const int32_t* vec, int k, uint32_t* res_idx, int32_t* res_val) {
  std::vector<unsigned> s(row, row + nnz), e(col, col + nnz);
  std::vector<int32_t> v(val, val + nnz);
  coo_t<unsigned, int32_t> coo(s, e, v);
  spmv_coo_gold_top_k_2<unsigned, int32_t, int32_t>(coo, const_cast<int32_t*>(vec), k, res_idx,
                                                    res_val);
}

void ref_gold_topk_f32(const uint32_t* row, const uint32_t* col, const float* val, uint64_t nnz,
                       const float* vec, int k, uint32_t* res_idx, float* res_val) {
  std::vector<unsigned> s(row, row + nnz), e(col, col + nnz);
  std::vector<float> v(val, val + nnz);
  coo_t<unsigned, float> coo(s, e, v);
  spmv_coo_gold_top_k<unsigned, float>(coo, const_cast<float*>(vec), k, res_idx, res_val);
}

void ref_gold4_f32(const uint32_t* row, const uint32_t* col, const float* val, uint64_t nnz,
                   const float* vec, uint32_t rows, float* result) {
  std::vector<unsigned> s(row, row + nnz), e(col, col + nnz);
  std::vector<float> v(val, val + nnz);
  coo_t<unsigned, float> coo(s, e, v);
  for (uint32_t i = 0; i < rows; i++) result[i] = 0.0f;
  spmv_coo_gold4<unsigned, float>(coo, result, const_cast<float*>(vec));
}

void ref_sort_tuples_f32(uint32_t n, uint32_t* idx, float* val) {
  sort_tuples<uint32_t, float>(n, idx, val);
}

void ref_sort_tuples_i32(uint32_t n, uint32_t* idx, int32_t* val) {
  sort_tuples<uint32_t, int32_t>(n, idx, val);
}

void ref_sort_pr_f32(uint32_t n, const float* val, uint32_t* out_idx) {
  std::vector<index_type> o = sort_pr<float>(n, const_cast<float*>(val));
  for (uint32_t i = 0; i < n; i++) out_idx[i] = o[i];
}

/* readMtx into caller arrays of capacity cap; returns the entry count (0 when over cap).
 * The reference exits the process on a malformed file: call it on valid files only. */
uint32_t ref_read_mtx(const char* path, int directed, int read_values, int zero_indexed,
                      int sort, uint32_t* rows, uint32_t* cols, uint32_t* row, uint32_t* col,
                      float* val, uint32_t cap) {
  std::vector<unsigned> r, c;
  std::vector<float> v;
  unsigned nr = 0, nc = 0, nz = 0;
  readMtx<unsigned, float>(path, &r, &c, &v, &nr, &nc, &nz, directed, read_values != 0, false,
                           zero_indexed != 0, sort != 0);
  *rows = nr;
  *cols = nc;
  if (r.size() > cap) return 0;
  for (size_t i = 0; i < r.size(); i++) {
    row[i] = r[i];
    col[i] = c[i];
    val[i] = v[i];
  }
  return (uint32_t)r.size();
}

}  // extern "C"
