// aes_gpu_baseline.cu -- the reference's GPU comparison path, for timing only: a library
// SpMV over the FP32 CSR (cuSPARSE), then a full descending sort of all row scores, then the
// first K (reference: src/gpu/host_spmv_topk_csr_gpu_int8.cu SpMV :68-314 -- cusparseSpMV,
// thrust::sort_by_key over every row, get_topk).  Not part of the Top-K path: no low-bit stage,
// and equal scores come out in ascending row order (a stable radix sort), not the path's
// (score desc, row desc).
#include <cuda_runtime.h>
#include <cusparse.h>

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <string>
#include <vector>

#include "acceles.h"
#include "aes_host.hpp"

namespace aes {
const char* last_error_cstr();
}

namespace {

__global__ void k_iota(uint32_t* p, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = i;
}

struct Scratch {
  std::vector<void*> ptrs;
  cusparseHandle_t sp = nullptr;
  cusparseSpMatDescr_t A = nullptr;
  cusparseDnVecDescr_t x = nullptr, y = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t s = nullptr;
  ~Scratch() {
    if (A) cusparseDestroySpMat(A);
    if (x) cusparseDestroyDnVec(x);
    if (y) cusparseDestroyDnVec(y);
    if (sp) cusparseDestroy(sp);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** p, size_t n) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n * sizeof(T), 16));
    if (e == cudaSuccess) {
      ptrs.push_back(q);
      *p = static_cast<T*>(q);
    }
    return e;
  }
};

}  // namespace

#define BL_CK(x)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (x);                                                                     \
    if (e_ != cudaSuccess) {                                                                  \
      cudaGetLastError();                                                                     \
      return aes::fail(AES_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));       \
    }                                                                                         \
  } while (0)
#define BL_SP(x)                                                                              \
  do {                                                                                        \
    cusparseStatus_t s_ = (x);                                                                \
    if (s_ != CUSPARSE_STATUS_SUCCESS)                                                        \
      return aes::fail(AES_ERR_CUDA, std::string(#x) + ": " + cusparseGetErrorString(s_));    \
  } while (0)

extern "C" int aes_baseline_cusparse_topk(const uint64_t* ptr, const uint32_t* col,
                                          const float* val, uint32_t rows, uint32_t cols,
                                          const float* queries, uint32_t nq, uint32_t k,
                                          int device, uint32_t* out_idx, float* out_score,
                                          double* ms_per_query) {
  if (!ptr || !queries || !out_idx || !out_score || !ms_per_query)
    return aes::fail(AES_ERR_INVALID, "NULL argument");
  if (rows == 0 || cols == 0 || k == 0 || k > rows || nq == 0)
    return aes::fail(AES_ERR_INVALID, "empty shape, k or batch");
  const uint64_t nnz = ptr[rows];
  if (nnz >= 0x7FFFFFFFull || rows >= 0x7FFFFFFFu)
    return aes::fail(AES_ERR_UNSUPPORTED, "32-bit cuSPARSE indices");
  if (nnz && (!col || !val)) return aes::fail(AES_ERR_INVALID, "NULL CSR array");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return aes::fail(AES_ERR_NODEV, "no CUDA device");
  }
  BL_CK(cudaSetDevice(device));
  Scratch S;
  BL_CK(cudaStreamCreateWithFlags(&S.s, cudaStreamNonBlocking));
  BL_CK(cudaEventCreate(&S.e0));
  BL_CK(cudaEventCreate(&S.e1));
  int32_t *d_ptr = nullptr, *d_col = nullptr;
  float *d_val = nullptr, *d_x = nullptr, *d_y = nullptr, *d_ky = nullptr;
  uint32_t *d_i0 = nullptr, *d_i1 = nullptr;
  BL_CK(S.alloc(&d_ptr, (size_t)rows + 1));
  BL_CK(S.alloc(&d_col, nnz));
  BL_CK(S.alloc(&d_val, nnz));
  BL_CK(S.alloc(&d_x, cols));
  BL_CK(S.alloc(&d_y, rows));
  BL_CK(S.alloc(&d_ky, rows));
  BL_CK(S.alloc(&d_i0, rows));
  BL_CK(S.alloc(&d_i1, rows));
  {
    std::vector<int32_t> p32((size_t)rows + 1), c32(nnz);
    for (uint32_t r = 0; r <= rows; r++) p32[r] = (int32_t)ptr[r];
    for (uint64_t i = 0; i < nnz; i++) c32[i] = (int32_t)col[i];
    BL_CK(cudaMemcpy(d_ptr, p32.data(), p32.size() * 4, cudaMemcpyHostToDevice));
    if (nnz) {
      BL_CK(cudaMemcpy(d_col, c32.data(), nnz * 4, cudaMemcpyHostToDevice));
      BL_CK(cudaMemcpy(d_val, val, nnz * 4, cudaMemcpyHostToDevice));
    }
  }
  BL_SP(cusparseCreate(&S.sp));
  BL_SP(cusparseSetStream(S.sp, S.s));
  BL_SP(cusparseCreateCsr(&S.A, rows, cols, (int64_t)nnz, d_ptr, d_col, d_val, CUSPARSE_INDEX_32I,
                          CUSPARSE_INDEX_32I, CUSPARSE_INDEX_BASE_ZERO, CUDA_R_32F));
  BL_SP(cusparseCreateDnVec(&S.x, cols, d_x, CUDA_R_32F));
  BL_SP(cusparseCreateDnVec(&S.y, rows, d_y, CUDA_R_32F));
  const float alpha = 1.0f, beta = 0.0f;
  size_t spbytes = 0, sortbytes = 0;
  BL_SP(cusparseSpMV_bufferSize(S.sp, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, S.A, S.x, &beta,
                                S.y, CUDA_R_32F, CUSPARSE_SPMV_ALG_DEFAULT, &spbytes));
  BL_CK(cub::DeviceRadixSort::SortPairsDescending(nullptr, sortbytes, d_y, d_ky, d_i0, d_i1,
                                                  (int)rows, 0, 32, S.s));
  unsigned char *d_spbuf = nullptr, *d_sortbuf = nullptr;
  BL_CK(S.alloc(&d_spbuf, spbytes));
  BL_CK(S.alloc(&d_sortbuf, sortbytes));
  double total_ms = 0.0;
  for (uint32_t q = 0; q < nq; q++) {
    BL_CK(cudaMemcpyAsync(d_x, queries + (size_t)q * cols, cols * 4ull, cudaMemcpyHostToDevice, S.s));
    BL_CK(cudaEventRecord(S.e0, S.s));
    BL_SP(cusparseSpMV(S.sp, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, S.A, S.x, &beta, S.y,
                       CUDA_R_32F, CUSPARSE_SPMV_ALG_DEFAULT, d_spbuf));
    k_iota<<<1024, 256, 0, S.s>>>(d_i0, rows);
    BL_CK(cudaGetLastError());
    BL_CK(cub::DeviceRadixSort::SortPairsDescending(d_sortbuf, sortbytes, d_y, d_ky, d_i0, d_i1,
                                                    (int)rows, 0, 32, S.s));
    BL_CK(cudaEventRecord(S.e1, S.s));
    BL_CK(cudaMemcpyAsync(out_idx + (size_t)q * k, d_i1, k * 4ull, cudaMemcpyDeviceToHost, S.s));
    BL_CK(cudaMemcpyAsync(out_score + (size_t)q * k, d_ky, k * 4ull, cudaMemcpyDeviceToHost, S.s));
    BL_CK(cudaStreamSynchronize(S.s));
    float ms = 0.0f;
    BL_CK(cudaEventElapsedTime(&ms, S.e0, S.e1));
    if (q > 0 || nq == 1) total_ms += ms;  // the first query warms the library up
  }
  *ms_per_query = total_ms / (nq > 1 ? nq - 1 : 1);
  return AES_OK;
}

extern "C" const char* aes_baseline_last_error(void) { return aes::last_error_cstr(); }
