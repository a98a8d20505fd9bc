// acceles_spmv.hpp -- C++ drop-in for the reference's quantised host driver `struct SpMV`
// (zhaijiaqi/AccelES, src/fpga/src/host_spmv_ucsr.cpp:134-829), header-only over the C ABI of
// acceles.h.  Method names, argument meaning and call order follow the reference so that a
// main() shaped like host_spmv_ucsr.cpp:894-1193 drives the GB300 engine:
//
//   aes::SpMV q_spmv(x, y, val, rows, cols, nnz, vec, debug);   // :1066 (packs + uploads)
//   q_spmv.Q_reset(vec, debug);                                  // :1113 (new query)
//   long ns = q_spmv(true, debug);                               // :1099 (run, device ns)
//   q_spmv.Q_read_result(res, idx, debug);                       // :1106 (merged candidates)
//
// Two constructors: the reference's quantised one (pre-quantised COO values q_val and query q_vec,
// as the reference's own main reads them from a _quantified_B*.mtx file, :969-977), and one taking
// the FP32 COO, which the engine quantises itself and keeps for the exact pass.  Q_reset takes
// either a quantised (int8) or an FP32 query.  The quantised constructor turns on Q_read_result's
// filter of non-positive candidates (:709) unless params say otherwise.  Errors throw aes::Error
// instead of exiting (OCL_CHECK, opencl_utils.hpp:27-33); read_topk() adds the final Top-K, FP32-
// rescored when FP32 values are at hand, which the reference computes only in its Python scripts
// (quantify_util.py:332-372).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "acceles.h"

namespace aes {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error("[" + std::to_string(c) + "] " + m), code(c) {}
};

inline void check(int rc) {
  if (rc != AES_OK) throw Error(rc, aes_last_error());
}

class SpMV {
 public:
  // rows/cols/nnz and the COO arrays as in the quantised constructor (:198); `vec` (may be
  // null) is the first query, of length cols.
  SpMV(const uint32_t* x, const uint32_t* y, const float* val, uint32_t rows, uint32_t cols,
       uint64_t nnz, const float* vec = nullptr, int debug = 0,
       const aes_params* params = nullptr)
      : cols_(cols) {
    (void)debug;
    aes_params p;
    if (params) p = *params;
    else aes_params_default(&p);
    check(aes_create(x, y, val, rows, cols, nnz, &p, &h_));
    k_ = p.k_max;
    if (vec) Q_reset(vec, 0);
  }
  // The quantised constructor SpMV(ConfigOpenCL&, q_x, q_y, q_val, rows, cols, nnz, q_vec,
  // debug) (:198-218): q_val holds B-bit signed values, q_vec (may be null) the first quantised
  // query; val_f32 (may be null) the FP32 values of the same entries for an exact pass.
  SpMV(const uint32_t* q_x, const uint32_t* q_y, const int8_t* q_val, uint32_t rows,
       uint32_t cols, uint64_t nnz, const int8_t* q_vec, int debug = 0,
       const aes_params* params = nullptr, const float* val_f32 = nullptr)
      : cols_(cols) {
    (void)debug;
    aes_params p;
    if (params) p = *params;
    else {
      aes_params_default(&p);
      p.flags |= AES_FLAG_POSITIVE;
    }
    check(aes_create_quantized(q_x, q_y, q_val, val_f32, rows, cols, nnz, &p, &h_));
    k_ = p.k_max;
    if (q_vec) Q_reset(q_vec, 0);
  }
  SpMV(const SpMV&) = delete;
  SpMV& operator=(const SpMV&) = delete;
  SpMV(SpMV&& o) noexcept : h_(std::exchange(o.h_, nullptr)), cols_(o.cols_), k_(o.k_), nq_(o.nq_) {}
  ~SpMV() { aes_destroy(h_); }

  // Q_reset (:790-828): load a new query (or nq queries, row-major); returns host ns.
  long Q_reset(const float* vec, int debug = 0, uint32_t nq = 1) {
    (void)debug;
    check(aes_set_query(h_, vec, nq));
    nq_ = nq;
    return 0;
  }

  // Q_reset(q_type* vec, int debug) (:790-828) with the reference's quantised query (or nq of
  // them); q_f32 (may be null) the same queries in FP32 for the exact pass.
  long Q_reset(const int8_t* vec, int debug = 0, uint32_t nq = 1, const float* q_f32 = nullptr) {
    (void)debug;
    check(aes_set_query_quantized(h_, vec, q_f32, nq));
    nq_ = nq;
    return 0;
  }

  // operator()(bool, int) (:556-565): run the loaded queries, wait, return device ns.
  long operator()(bool flag = true, int debug = 0) {
    (void)flag;
    (void)debug;
    idx_.assign((size_t)nq_ * k_, 0);
    score_.assign((size_t)nq_ * k_, 0.0f);
    uint64_t ns = 0;
    check(aes_run(h_, k_, idx_.data(), score_.data(), &ns));
    return (long)ns;
  }

  // Q_read_result (:691-748): append the candidates of query `query`, sorted by (integer score
  // descending, row descending) as sort_tuples orders them.
  void Q_read_result(std::vector<int32_t>& res, std::vector<uint32_t>& idx, int debug = 0,
                     uint32_t query = 0) {
    (void)debug;
    aes_info inf;
    check(aes_get_info(h_, &inf));
    std::vector<uint32_t> i(inf.ck);
    std::vector<int32_t> s(inf.ck);
    uint32_t n = 0;
    check(aes_read_candidates(h_, query, i.data(), s.data(), nullptr, inf.ck, &n));
    if (n > inf.ck) n = inf.ck;
    idx.insert(idx.end(), i.begin(), i.begin() + n);
    res.insert(res.end(), s.begin(), s.begin() + n);
  }

  // Final FP32 Top-K of the last run: rows and scores of query `query` (k_max entries).
  std::pair<std::vector<uint32_t>, std::vector<float>> read_topk(uint32_t query = 0) const {
    auto b = idx_.begin() + (size_t)query * k_;
    auto c = score_.begin() + (size_t)query * k_;
    return {std::vector<uint32_t>(b, b + k_), std::vector<float>(c, c + k_)};
  }

  aes_handle* handle() const { return h_; }

 private:
  aes_handle* h_ = nullptr;
  uint32_t cols_ = 0, k_ = 0, nq_ = 0;
  std::vector<uint32_t> idx_;
  std::vector<float> score_;
};

}  // namespace aes
