// aes_engine.cu -- the device-resident Top-K SpMV engine behind the C ABI of include/acceles.h.
//
// One handle = one matrix resident in HBM (Ultra-CSR tiles + FP32 CSR) plus per-batch buffers.
// A run enqueues, on the handle's stream:
//   k_quantize -> k_cand_plain(sample tiles) -> k_threshold -> k_cand_plain(all tiles, filter)
//   -> k_select -> k_final
// and afterwards repairs, on the exact slow path, any query whose sample threshold missed or
// whose survivor buffer overflowed (status bits).  Reference host API replaced:
// struct SpMV, src/fpga/src/host_spmv_ucsr.cpp:134-829 (zhaijiaqi/AccelES).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "acceles.h"
#include "aes_host.hpp"
#include "aes_kernels.cuh"
#include "aes_select.cuh"
#include "aes_batch.cuh"
#include "aes_tc.cuh"

namespace aes {
const char* last_error_cstr();

#define AES_CK(x)                                                                            \
  do {                                                                                       \
    cudaError_t e_ = (x);                                                                    \
    if (e_ != cudaSuccess) return ::aes::fail(AES_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

using namespace dev;

typedef void (*PlainKernel)(PlainArgs);
typedef void (*BatchKernel)(BatchArgs);

template <int B, bool SGN>
static BatchKernel batch_kernel(int mode) {
  return mode == MODE_SAMPLE ? k_cand_batch<B, SGN, MODE_SAMPLE> : k_cand_batch<B, SGN, MODE_FILTER>;
}

static BatchKernel pick_batch(int bits, bool sgn, int mode) {
  switch (bits) {
    case 4: return sgn ? batch_kernel<4, true>(mode) : batch_kernel<4, false>(mode);
    case 6: return sgn ? batch_kernel<6, true>(mode) : batch_kernel<6, false>(mode);
    default: return sgn ? batch_kernel<8, true>(mode) : batch_kernel<8, false>(mode);
  }
}

template <int B, bool SGN>
static PlainKernel plain_kernel(int mode) {
  switch (mode) {
    case MODE_FILTER: return k_cand_plain<B, SGN, MODE_FILTER>;
    case MODE_SAMPLE: return k_cand_plain<B, SGN, MODE_SAMPLE>;
    default: return k_cand_plain<B, SGN, MODE_ALL>;
  }
}

static PlainKernel pick_plain(int bits, bool sgn, int mode) {
  switch (bits) {
    case 4: return sgn ? plain_kernel<4, true>(mode) : plain_kernel<4, false>(mode);
    case 6: return sgn ? plain_kernel<6, true>(mode) : plain_kernel<6, false>(mode);
    default: return sgn ? plain_kernel<8, true>(mode) : plain_kernel<8, false>(mode);
  }
}

static uint32_t pow2_at_least(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

// P(Bin(n, f) >= r) in log space
static double binom_tail(uint32_t n, double f, uint32_t r) {
  if (r == 0) return 1.0;
  if (r > n) return 0.0;
  if (f <= 0.0) return 0.0;
  if (f >= 1.0) return 1.0;
  double lf = std::log(f), l1f = std::log1p(-f), s = 0.0;
  for (uint32_t k = r; k <= n; k++) {
    double lt = std::lgamma((double)n + 1) - std::lgamma((double)k + 1) -
                std::lgamma((double)(n - k) + 1) + k * lf + (n - k) * l1f;
    s += std::exp(lt);
  }
  return s;
}

// Device arrays of a resident matrix (Ultra-CSR tiles, row bases, row scales, FP32 CSR,
// tensor-core layout), shared by a handle and the views made from it: freed with the last of them.
struct SharedAllocs {
  int device = -1;
  std::vector<void*> ptrs;
  ~SharedAllocs() {
    if (device >= 0) cudaSetDevice(device);
    for (void* p : ptrs) cudaFree(p);
  }
};

struct Engine {
  aes_params prm{};
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int sm_count = 0;

  uint32_t rows = 0, cols = 0, bits = 0, quant = 0, P = 0;
  uint64_t nnz = 0, qnnz = 0, packets = 0, tiles = 0;
  bool sgn = true;

  uint4* d_tiles = nullptr;
  uint32_t* d_tile_rowbase = nullptr;
  float* d_rowscale = nullptr;
  // tensor-core layout of a 4-bit matrix (AES_FLAG_TENSOR at creation)
  uint32_t* d_tc_ptr = nullptr;
  uint32_t* d_tc_ent = nullptr;
  uint32_t tc_nch = 0, tc_rtiles = 0;
  bool tc_ready = false;
  uint32_t* d_csr_ptr = nullptr;
  uint16_t* d_csr_col = nullptr;
  float* d_csr_val = nullptr;
  bool has_f32 = true;  // FP32 values resident: the exact pass can run

  // ---- configuration: selection geometry and per-batch buffers (aes_retune may change these) --
  struct Config {
    aes_params p{};
    uint32_t split = 1, slice = 0, ntop = 0, nslots = 0, ck_eff = 0, cap = 0;
    uint32_t ss = 1, n_sample_tiles = 0, n_sample_rows = 0, maxB = 1;
    std::vector<uint32_t> sample_first, part_begin, part_r;
    size_t plan = 0;  // device bytes of the configuration's buffers
  };
  Config cur;
  bool configured = false;

  uint32_t ss = 1, n_sample_tiles = 0, n_sample_rows = 0;
  uint32_t* d_sample_first = nullptr;
  uint32_t* d_part_sample_begin = nullptr;
  uint32_t* d_part_r = nullptr;

  uint32_t split = 1, slice = 0, ntop = 0, nslots = 0, ck_eff = 0, cap = 0;

  uint32_t maxB = 1, ld32 = 0, ld8 = 0;
  float* d_q32 = nullptr;
  int8_t* d_q8 = nullptr;
  uint32_t* d_sample_keys = nullptr;
  uint32_t* d_keys_t = nullptr;   // batched sample keys moved to [query][sample rows]
  uint32_t* d_exact_aux = nullptr;  // FP32-only pass: sample range {0, n} and rank r
  uint32_t* d_thr = nullptr;
  uint32_t* d_cnt = nullptr;
  uint2* d_surv = nullptr;
  uint32_t* d_cand = nullptr;
  uint32_t* d_cand_key = nullptr;
  uint32_t* d_status = nullptr;
  uint32_t* d_out_idx = nullptr;
  float* d_out_score = nullptr;
  uint32_t* d_allkeys = nullptr;
  uint32_t* d_exact_cand = nullptr;  // [k_max] candidates of the FP32-only pass
  uint32_t* d_exact_key = nullptr;

  float* h_q32 = nullptr;         // pinned staging of queries
  int8_t* h_q8 = nullptr;         // pinned staging of pre-quantised queries
  uint32_t* h_status = nullptr;   // pinned
  uint32_t nq_loaded = 0;
  bool q_pre = false;             // the loaded queries were given quantised
  bool q32_given = true;          // ... with their FP32 values (for the exact pass)
  bool last_int_final = false;    // the last run ranked its candidates by integer score
  uint32_t last_nq = 0, last_k = 0;
  bool last_from_device = false;
  const float* last_q32 = nullptr;   // query buffer of the last run
  uint32_t* last_idx = nullptr;      // device outputs of the last run
  float* last_score = nullptr;
  cudaStream_t last_stream = nullptr;
  bool ran = false;

  // CUDA graphs of the per-batch launch sequence, keyed by its arguments
  struct GraphKey {
    const float* q;
    uint32_t nq, k;
    uint32_t* idx;
    float* score;
    cudaStream_t s;
    bool pre;
    bool operator<(const GraphKey& o) const {
      return std::tie(q, nq, k, idx, score, s, pre) <
             std::tie(o.q, o.nq, o.k, o.idx, o.score, o.s, o.pre);
    }
  };
  std::map<GraphKey, cudaGraphExec_t> graphs;
  uint64_t n_graph_launch = 0;
  uint64_t graph_launches = 0, graph_cands = 0;  // kernels inside the last captured graph

  // profiling / counters
  uint64_t n_launch = 0, n_cand = 0, n_repaired = 0;
  std::vector<cudaEvent_t> prof_ev;  // pairs
  size_t prof_used = 0;
  double prof_ms = 0.0;
  uint64_t prof_n = 0;

  int plain_grid = 0, smem_optin = 0;
  size_t plain_smem = 0, final_smem = 0;
  // batched pass
  uint32_t* d_qtab = nullptr;     // [blocks][batch_qtab_words(cols)] words
  int batch_warps_n = 0, batch_grid = 0;
  size_t batch_smem = 0;
  uint32_t batch_mode = 0;        // 0 auto, 1 never, else always
  bool use_tc = false;            // batched candidate pass on the tensor cores
  uint8_t* d_qtab_tc = nullptr;   // [blocks][tc_qtab_bytes(cols)] e4m3 query operands
  size_t tc_smem = 0;
  int tc_grid = 0;
  uint32_t tc_nb = 2;  // chunk buffers of the tensor-core pass (tc_bufs)
  // the CTA-pair form (two 128-query blocks per launch), where a pair's shared memory fits and
  // clusters of two CTAs of that size can be scheduled
  bool tc_pair = false;
  size_t tc_smem2 = 0;
  int tc_grid2 = 0;
  uint32_t tc_nb2 = 2;
  bool last_batched = false;
  std::vector<uint32_t> h_tile_rowbase;  // host copy: sample geometry is derived from it
  size_t bytes = 0, mat_bytes = 0, cfg_bytes = 0;
  std::vector<void*> allocs, cfg_allocs;  // this handle's own arrays
  std::shared_ptr<SharedAllocs> mat_store;  // the matrix arrays, shared with views

  ~Engine() { release(); }

  void drop_graphs() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    graphs.clear();
  }

  void free_config() {
    drop_graphs();
    for (void* p : cfg_allocs) cudaFree(p);
    cfg_allocs.clear();
    if (h_q32) cudaFreeHost(h_q32);
    if (h_q8) cudaFreeHost(h_q8);
    if (h_status) cudaFreeHost(h_status);
    h_q32 = nullptr;
    h_q8 = nullptr;
    h_status = nullptr;
    d_sample_first = d_part_sample_begin = d_part_r = nullptr;
    d_q32 = nullptr;
    d_q8 = nullptr;
    d_sample_keys = d_keys_t = d_thr = d_cnt = d_cand = d_cand_key = d_status = d_out_idx = nullptr;
    d_surv = nullptr;
    d_out_score = nullptr;
    d_exact_cand = d_exact_key = d_qtab = d_exact_aux = nullptr;
    bytes -= cfg_bytes;
    cfg_bytes = 0;
    configured = false;
    nq_loaded = 0;
    ran = false;
    last_from_device = false;
  }

  void release() {
    if (device >= 0) cudaSetDevice(device);
    for (cudaEvent_t ev : prof_ev) cudaEventDestroy(ev);
    prof_ev.clear();
    free_config();
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    mat_store.reset();
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
    ev0 = ev1 = nullptr;
    stream = nullptr;
  }

  template <class T>
  int dalloc(T** p, size_t n, bool cfg = false) {
    size_t b = std::max<size_t>(n * sizeof(T), 16);
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(AES_ERR_NOMEM, std::string("cudaMalloc refused: ") + cudaGetErrorString(e));
    }
    (cfg ? cfg_allocs : allocs).push_back(q);
    (cfg ? cfg_bytes : mat_bytes) += b;
    bytes += b;
    *p = reinterpret_cast<T*>(q);
    return AES_OK;
  }

  int build(const HostCSR& m, const aes_params& p);
  int build_view(const Engine& base, const aes_params& p);
  int plan_config(const aes_params& p, Config* c) const;
  int apply_config(const Config& c);
  int retune(const aes_params& p);
  // d_q: the FP32 queries, or null when there are none (pre-quantised queries alone); pre: the
  // quantised queries are already in d_q8
  int enqueue(const float* d_q, uint32_t nq, uint32_t k, uint32_t* d_idx, float* d_score,
              cudaStream_t s, bool pre = false);
  int enqueue_graph(const float* d_q, uint32_t nq, uint32_t k, uint32_t* d_idx, float* d_score,
                    cudaStream_t s, bool pre = false);
  // the final Top-K ranks the candidates by integer score: no FP32 values or no FP32 queries
  bool int_final(const float* d_q) const { return !has_f32 || d_q == nullptr; }
  int repair(uint32_t nq, uint32_t k, uint32_t* d_idx, float* d_score, cudaStream_t s,
             uint32_t* repaired);
  int run_plain(int mode, uint32_t q, cudaStream_t s, uint32_t nq_y = 1);
  int run_batch(int mode, uint32_t nq, cudaStream_t s, uint32_t blk0 = 0, uint32_t nblk = 0);
  int run_tc(uint32_t blk, uint32_t nq_blk, cudaStream_t s, bool pair);
  int prof_open(cudaStream_t s);
  int prof_close(cudaStream_t s);
  int collect_profile();
  // the tensor-core pass serves a configuration: 4-bit layout built, flag set, thresholds of
  // every partition in shared memory, batched passes allowed
  bool tc_usable(const aes_params& p, uint32_t S) const {
    return tc_ready && (p.flags & AES_FLAG_TENSOR) && S <= kTcMaxSplit && p.batch_tile != 1 &&
           tc_smem_bytes(cols, S, 2, false) <= (size_t)smem_optin;
  }
};

// CUDA events around one full candidate-pass launch (AES_FLAG_PROFILE)
int Engine::prof_open(cudaStream_t s) {
  if (prof_used + 2 > prof_ev.size()) {
    if (prof_ev.size() >= 8192) {
      int rc = collect_profile();
      if (rc) return rc;
    } else {
      for (int i = 0; i < 256; i++) {
        cudaEvent_t ev;
        AES_CK(cudaEventCreate(&ev));
        prof_ev.push_back(ev);
      }
    }
  }
  AES_CK(cudaEventRecord(prof_ev[prof_used], s));
  return AES_OK;
}
int Engine::prof_close(cudaStream_t s) {
  AES_CK(cudaEventRecord(prof_ev[prof_used + 1], s));
  prof_used += 2;
  return AES_OK;
}

// Batched candidate pass on the tensor cores (aes_tc.cuh) of one block of <= 128 queries, or
// (pair) of blocks blk and blk + 1 (<= 256 queries) by CTA pairs; its query blocks are those of
// the dp4a pass, whose sample pass it shares
static_assert(kTcQ == kBatchQ, "tensor-core and dp4a passes use the same query blocks");
int Engine::run_tc(uint32_t blk, uint32_t nq_blk, cudaStream_t s, bool pair) {
  TcArgs a{};
  a.ent = d_tc_ent;
  a.ptr = d_tc_ptr;
  a.n_rtiles = tc_rtiles;
  a.nch = tc_nch;
  a.kpad = tc_kpad(cols);
  a.n_rows = rows;
  a.qt = d_qtab_tc + (size_t)blk * tc_qtab_bytes(cols);
  a.q0 = blk * kTcQ;
  a.nq = nq_blk;
  a.rowscale = d_rowscale;
  a.split = split;
  a.slice = slice;
  a.thr = d_thr;
  a.cnt = d_cnt;
  a.surv = d_surv;
  a.cap = cap;
  a.status = d_status;
  a.mma_idle = (prm.flags & AES_FLAG_TEST_IDLE_MMA) ? 1u : 0u;
  const bool prof = (prm.flags & AES_FLAG_PROFILE) != 0;
  int rc = prof ? prof_open(s) : AES_OK;
  if (rc) return rc;
  if (pair) {  // clusters of two CTAs: a pair per two SMs
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)tc_grid2);
    cfg.blockDim = dim3(kTcThreads);
    cfg.dynamicSmemBytes = tc_smem2;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    AES_CK(tc_nb2 == 3 ? cudaLaunchKernelEx(&cfg, k_cand_tc<3, true>, a)
                       : cudaLaunchKernelEx(&cfg, k_cand_tc<2, true>, a));
  } else if (tc_nb == 3) {
    k_cand_tc<3, false><<<tc_grid, kTcThreads, tc_smem, s>>>(a);
  } else {
    k_cand_tc<2, false><<<tc_grid, kTcThreads, tc_smem, s>>>(a);
  }
  AES_CK(cudaGetLastError());
  if (prof && (rc = prof_close(s))) return rc;
  n_launch++;
  n_cand++;
  return AES_OK;
}

int Engine::collect_profile() {
  for (size_t i = 0; i + 1 < prof_used; i += 2) {
    AES_CK(cudaEventSynchronize(prof_ev[i + 1]));
    float ms = 0.0f;
    AES_CK(cudaEventElapsedTime(&ms, prof_ev[i], prof_ev[i + 1]));
    prof_ms += ms;
    prof_n++;
  }
  prof_used = 0;
  return AES_OK;
}

// Device bytes of the matrix itself: Ultra-CSR tiles, tile row bases, per-row scales, the FP32
// CSR of the exact pass and the slow path's key array.
static size_t matrix_plan(uint64_t tiles, uint32_t rows, uint64_t nnz, uint32_t quant,
                          bool has_f32) {
  size_t plan = tiles * (size_t)kTileBytes + (tiles + 1) * 4;
  plan += (quant == AES_QUANT_UNSIGNED_ROW) ? rows * 4ull : 0;
  plan += has_f32 ? (rows + 1) * 4ull + nnz * 6ull : 0;
  plan += rows * 4ull;
  return plan;
}

// Host-only: selection geometry, sample tiles, per-partition sample ranks and the device bytes
// of the configuration's buffers.  Needs rows, cols, tiles and h_tile_rowbase.
int Engine::plan_config(const aes_params& p, Config* c) const {
  c->p = p;
  const uint32_t S = p.split <= 1 ? 1 : p.split;
  c->split = S;
  c->slice = rows / S;
  c->ntop = p.ck / S;
  c->nslots = S * c->ntop;
  c->ck_eff = 0;
  std::vector<uint32_t> prow(S);
  for (uint32_t q = 0; q < S; q++) {
    uint32_t r0 = q * c->slice, r1 = (q == S - 1) ? rows : (q + 1) * c->slice;
    prow[q] = r1 - r0;
    c->ck_eff += std::min(c->ntop, prow[q]);
  }

  // sample tiles: every ss-th tile, with the rows each one owns
  // auto: every tile of a tiny matrix, else one tile in 64; one in 256 for a large matrix with
  // one partition.  Several partitions keep Top-(CK/split) each: the bound of so few candidates
  // from a sparse sample sits far below the boundary and lets many rows through to the survivor
  // buffers (10M x 1024, 8-bit, 32 partitions: 99 us per pass at one tile in 256, 85 us at 64)
  if (p.sample_stride) c->ss = p.sample_stride;
  else c->ss = tiles <= 64 ? 1 : ((tiles <= 16384 || S > 1) ? 64 : 256);
  const uint32_t ss_ = c->ss;
  c->n_sample_tiles = (uint32_t)((tiles + ss_ - 1) / ss_);
  auto owned_begin = [&](uint64_t t) -> uint64_t {
    if (t >= tiles) return rows;
    return t == 0 ? 0 : (uint64_t)h_tile_rowbase[t] + 1;
  };
  c->sample_first.assign(c->n_sample_tiles, 0);
  std::vector<uint64_t> s_begin(c->n_sample_tiles), s_end(c->n_sample_tiles);
  uint64_t pre = 0;
  for (uint32_t s = 0; s < c->n_sample_tiles; s++) {
    uint64_t t = (uint64_t)s * ss_;
    uint64_t b = owned_begin(t), e = std::max(b, owned_begin(t + 1));
    s_begin[s] = b;
    s_end[s] = e;
    c->sample_first[s] = (uint32_t)(b - pre);
    pre += e - b;
  }
  c->n_sample_rows = (uint32_t)pre;
  // sample index range of each partition
  c->part_begin.assign(S + 1, 0);
  {
    uint32_t s = 0;
    uint64_t idx = 0;  // sample rows before s_begin[s]
    for (uint32_t q = 0; q <= S; q++) {
      uint64_t rb = (q == S) ? rows : (uint64_t)q * c->slice;
      while (s < c->n_sample_tiles && s_end[s] <= rb) { idx += s_end[s] - s_begin[s]; s++; }
      uint64_t cc = idx;
      if (s < c->n_sample_tiles && s_begin[s] < rb) cc += rb - s_begin[s];
      c->part_begin[q] = (uint32_t)cc;
    }
    c->part_begin[S] = c->n_sample_rows;
  }
  // r = smallest rank whose binomial tail is below 1e-12: the r-th largest sample key is then
  // below the partition's ntop-th largest key except with that probability
  c->part_r.assign(S, 0);
  size_t cap_need = 1024;
  for (uint32_t q = 0; q < S; q++) {
    uint32_t ns = c->part_begin[q + 1] - c->part_begin[q];
    double f = prow[q] ? (double)ns / (double)prow[q] : 1.0;
    uint32_t n1 = c->ntop ? c->ntop - 1 : 0;
    uint32_t r = 1;
    if (f >= 1.0) r = std::max<uint32_t>(c->ntop, 1);
    else {
      r = (uint32_t)std::floor(n1 * f);
      while (r <= n1 && binom_tail(n1, f, r) > 1e-12) r++;
      r = std::max<uint32_t>(r, 1);
    }
    c->part_r[q] = r;
    double expect = f > 0 ? (double)r / f : (double)prow[q];
    size_t cc = (size_t)std::min<double>((double)prow[q], 4.0 * expect + 4.0 * c->ntop + 1024.0);
    cap_need = std::max(cap_need, cc);
  }
  c->cap = (uint32_t)std::min<size_t>(cap_need, (size_t)rows);
  if (c->cap == 0) c->cap = 1;

  c->maxB = std::max<uint32_t>(p.max_batch, 1);
  const size_t maxB = c->maxB;
  const size_t nblk = (maxB + kBatchQ - 1) / kBatchQ;
  size_t plan = (c->n_sample_tiles + 2ull * S + 2) * 4;
  plan += nblk * kBatchQ * (size_t)c->n_sample_rows * 4;
  plan += maxB * (size_t)c->n_sample_rows * 4;  // the same keys, query-major
  plan += maxB * (ld32 * 4ull + ld8 + S * 8ull + (size_t)S * c->cap * 8 + c->nslots * 8ull + 4 +
                  p.k_max * 8ull);
  plan += nblk * batch_qtab_words(cols) * 4;
  if (tc_usable(p, S)) plan += nblk * tc_qtab_bytes(cols);
  plan += p.k_max * 8ull;
  c->plan = plan;

  const size_t psmem = plain_smem_bytes((int)bits, cols, S);
  if (psmem > (size_t)smem_optin)
    return fail(AES_ERR_UNSUPPORTED, "shared memory of the candidate pass exceeds the device limit");
  return AES_OK;
}

// Allocates the configuration's buffers, uploads its sample metadata and sets launch geometry.
int Engine::apply_config(const Config& c) {
  split = c.split;
  slice = c.slice;
  ntop = c.ntop;
  nslots = c.nslots;
  ck_eff = c.ck_eff;
  cap = c.cap;
  ss = c.ss;
  n_sample_tiles = c.n_sample_tiles;
  n_sample_rows = c.n_sample_rows;
  maxB = c.maxB;
  const aes_params& p = c.p;

  int rc2 = 0;
#define AES_AL(ptr, n) if ((rc2 = dalloc(&(ptr), (n), true)) != AES_OK) return rc2
  AES_AL(d_sample_first, std::max<uint32_t>(n_sample_tiles, 1));
  AES_AL(d_part_sample_begin, split + 1);
  AES_AL(d_part_r, split);
  AES_AL(d_q32, (size_t)maxB * ld32);
  AES_AL(d_q8, (size_t)maxB * ld8);
  // batched passes write sample keys per block of kBatchQ queries: pad to whole blocks
  const size_t maxB_blk = (size_t)((maxB + kBatchQ - 1) / kBatchQ) * kBatchQ;
  AES_AL(d_sample_keys, maxB_blk * std::max<uint32_t>(n_sample_rows, 1));
  AES_AL(d_keys_t, (size_t)maxB * std::max<uint32_t>(n_sample_rows, 1));
  AES_AL(d_thr, (size_t)maxB * split);
  AES_AL(d_cnt, (size_t)maxB * split);
  AES_AL(d_surv, (size_t)maxB * split * cap);
  AES_AL(d_cand, (size_t)maxB * std::max<uint32_t>(nslots, 1));
  AES_AL(d_cand_key, (size_t)maxB * std::max<uint32_t>(nslots, 1));
  AES_AL(d_status, maxB);
  AES_AL(d_out_idx, (size_t)maxB * std::max<uint32_t>(p.k_max, 1));
  AES_AL(d_out_score, (size_t)maxB * std::max<uint32_t>(p.k_max, 1));
  AES_AL(d_qtab, (size_t)((maxB + kBatchQ - 1) / kBatchQ) * batch_qtab_words(cols));
  use_tc = tc_usable(p, split);
  if (use_tc) AES_AL(d_qtab_tc, (size_t)((maxB + kTcQ - 1) / kTcQ) * tc_qtab_bytes(cols));
  AES_AL(d_exact_cand, std::max<uint32_t>(p.k_max, 1));
  AES_AL(d_exact_key, std::max<uint32_t>(p.k_max, 1));
  AES_AL(d_exact_aux, 4);
#undef AES_AL
  AES_CK(cudaMallocHost(&h_q32, (size_t)maxB * ld32 * sizeof(float)));
  AES_CK(cudaMallocHost(&h_q8, (size_t)maxB * ld8));
  AES_CK(cudaMallocHost(&h_status, (size_t)maxB * sizeof(uint32_t)));
  if (n_sample_tiles)
    AES_CK(cudaMemcpy(d_sample_first, c.sample_first.data(), n_sample_tiles * 4ull, cudaMemcpyHostToDevice));
  AES_CK(cudaMemcpy(d_part_sample_begin, c.part_begin.data(), (split + 1) * 4ull, cudaMemcpyHostToDevice));
  AES_CK(cudaMemcpy(d_part_r, c.part_r.data(), split * 4ull, cudaMemcpyHostToDevice));
  AES_CK(cudaMemset(d_q32, 0, (size_t)maxB * ld32 * 4));

  // ---- launch geometry ---------------------------------------------------------------------
  plain_smem = plain_smem_bytes((int)bits, cols, split);
  int occ = 0;
  AES_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &occ, (const void*)pick_plain((int)bits, sgn, MODE_FILTER), plain_threads((int)bits), plain_smem));
  plain_grid = std::max(1, occ) * sm_count;
  batch_mode = p.batch_tile;
  batch_warps_n = batch_warps((int)bits, cols, split);  // the most that fit
  if (p.batch_warps && (int)p.batch_warps < batch_warps_n) batch_warps_n = (int)p.batch_warps;
  if (batch_warps_n < 1) batch_mode = 1;  // query table does not fit: plain passes only
  if (batch_mode != 1) {
    batch_smem = batch_smem_bytes((int)bits, cols, split, batch_warps_n);
    int occb = 0;
    AES_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occb, (const void*)pick_batch((int)bits, sgn, MODE_FILTER), batch_warps_n * 32, batch_smem));
    batch_grid = std::max(1, occb) * sm_count;
  }
  if (use_tc) {  // one CTA per SM (its shared memory), persistent over the 128-row tiles
    tc_nb = tc_bufs(cols, split, (size_t)smem_optin, false);
    tc_smem = tc_smem_bytes(cols, split, tc_nb, false);
    tc_grid = (int)std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)sm_count, tc_rtiles));
    tc_pair = false;
    if (tc_smem_bytes(cols, split, 2, true) <= (size_t)smem_optin && sm_count >= 2) {
      tc_nb2 = tc_bufs(cols, split, (size_t)smem_optin, true);
      tc_smem2 = tc_smem_bytes(cols, split, tc_nb2, true);
      const uint32_t pairs = std::max<uint32_t>(
          1, std::min<uint32_t>((uint32_t)sm_count / 2, (tc_rtiles + 1) / 2));
      tc_grid2 = 2 * (int)pairs;
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3((unsigned)tc_grid2);
      cfg.blockDim = dim3(kTcThreads);
      cfg.dynamicSmemBytes = tc_smem2;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = 2;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      const cudaError_t e = tc_nb2 == 3
          ? cudaOccupancyMaxActiveClusters(&nclusters, k_cand_tc<3, true>, &cfg)
          : cudaOccupancyMaxActiveClusters(&nclusters, k_cand_tc<2, true>, &cfg);
      if (e == cudaSuccess && nclusters > 0) tc_pair = true;
      else (void)cudaGetLastError();  // the single-CTA form serves every block
    }
  } else {
    d_qtab_tc = nullptr;
  }
  {
    uint32_t kp = 1;
    while (kp < p.k_max) kp <<= 1;
    final_smem = final_smem_bytes(cols, std::max(nslots, p.k_max), kp);
  }
  prm = p;
  cur = c;
  configured = true;
  return AES_OK;
}

int Engine::build(const HostCSR& m, const aes_params& p) {
  prm = p;
  device = p.device;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(AES_ERR_NODEV, "no CUDA device");
  }
  if (device < 0 || device >= ndev) return fail(AES_ERR_INVALID, "device ordinal out of range");
  AES_CK(cudaSetDevice(device));
  AES_CK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
  AES_CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  AES_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  AES_CK(cudaEventCreate(&ev0));
  AES_CK(cudaEventCreate(&ev1));

  rows = m.rows;
  cols = m.cols;
  bits = p.bits;
  quant = p.quant;
  sgn = (quant == AES_QUANT_SYM_GLOBAL);
  nnz = m.ptr[rows];
  has_f32 = !m.prequantized || m.val.size() == nnz;
  if (nnz >= 0xFFFFFFFFull) return fail(AES_ERR_UNSUPPORTED, "nnz must be below 2^32");
  ld32 = (cols + 3) & ~3u;
  ld8 = (cols + 15) & ~15u;

  PackedMatrix pm;
  int rc = quantize_and_pack(m, p, &pm);
  if (rc) return rc;
  P = pm.P;
  qnnz = pm.qnnz;
  packets = pm.packets;
  tiles = pm.tiles;
  if (tiles >= 0xFFFFFFFFull) return fail(AES_ERR_UNSUPPORTED, "matrix too large");
  h_tile_rowbase = pm.tile_rowbase;
  tc_ready = !pm.tc_ptr.empty();
  tc_nch = pm.tc_nch;
  tc_rtiles = (uint32_t)((rows + kTcRows - 1) / kTcRows);
  const size_t tc_bytes = tc_ready ? (pm.tc_ptr.size() + pm.tc_ent.size()) * 4 : 0;

  Config c;
  rc = plan_config(p, &c);
  if (rc) return rc;

  // ---- memory plan and admission: nothing is allocated unless all of it fits ---------------
  const size_t plan = matrix_plan(tiles, rows, nnz, quant, has_f32) + tc_bytes + c.plan;
  if (p.mem_limit && plan > p.mem_limit)
    return fail(AES_ERR_NOMEM, "matrix needs " + std::to_string(plan) +
                                   " device bytes, over the handle limit " +
                                   std::to_string(p.mem_limit));
  size_t freeb = 0, totalb = 0;
  AES_CK(cudaMemGetInfo(&freeb, &totalb));
  if (plan + (64ull << 20) > freeb)
    return fail(AES_ERR_NOMEM, "matrix needs " + std::to_string(plan) + " device bytes, " +
                                   std::to_string(freeb) + " free");

  int rc2 = 0;
#define AES_AL(ptr, n) if ((rc2 = dalloc(&(ptr), (n))) != AES_OK) return rc2
  AES_AL(d_tiles, tiles * 128);
  AES_AL(d_tile_rowbase, tiles + 1);
  if (quant == AES_QUANT_UNSIGNED_ROW) AES_AL(d_rowscale, rows);
  if (has_f32) {
    AES_AL(d_csr_ptr, rows + 1);
    AES_AL(d_csr_col, std::max<uint64_t>(nnz, 1));
    AES_AL(d_csr_val, std::max<uint64_t>(nnz, 1));
  }
  AES_AL(d_allkeys, rows);
  if (tc_ready) {
    AES_AL(d_tc_ptr, pm.tc_ptr.size());
    AES_AL(d_tc_ent, std::max<size_t>(pm.tc_ent.size(), 1));
  }
#undef AES_AL

  // ---- upload -----------------------------------------------------------------------------------
  std::vector<uint32_t> ptr32(has_f32 ? rows + 1 : 0);
  std::vector<uint16_t> col16(has_f32 ? nnz : 0);
  if (has_f32) {
    for (uint32_t r = 0; r <= rows; r++) ptr32[r] = (uint32_t)m.ptr[r];
    parallel_for(nnz, 1 << 20, [&](uint64_t b, uint64_t e) {
      for (uint64_t i = b; i < e; i++) col16[i] = (uint16_t)m.col[i];
    });
  }
  AES_CK(cudaMemcpy(d_tiles, pm.tile_bytes.data(), pm.tile_bytes.size(), cudaMemcpyHostToDevice));
  AES_CK(cudaMemcpy(d_tile_rowbase, pm.tile_rowbase.data(), (tiles + 1) * 4, cudaMemcpyHostToDevice));
  if (d_rowscale) AES_CK(cudaMemcpy(d_rowscale, pm.rowscale.data(), rows * 4ull, cudaMemcpyHostToDevice));
  if (has_f32) AES_CK(cudaMemcpy(d_csr_ptr, ptr32.data(), (rows + 1) * 4ull, cudaMemcpyHostToDevice));
  if (has_f32 && nnz) {
    AES_CK(cudaMemcpy(d_csr_col, col16.data(), nnz * 2, cudaMemcpyHostToDevice));
    AES_CK(cudaMemcpy(d_csr_val, m.val.data(), nnz * 4, cudaMemcpyHostToDevice));
  }
  if (tc_ready) {
    AES_CK(cudaMemcpy(d_tc_ptr, pm.tc_ptr.data(), pm.tc_ptr.size() * 4, cudaMemcpyHostToDevice));
    if (!pm.tc_ent.empty())
      AES_CK(cudaMemcpy(d_tc_ent, pm.tc_ent.data(), pm.tc_ent.size() * 4, cudaMemcpyHostToDevice));
  }

  // the shared-memory limit is an attribute of the kernel, shared by every handle: raise it to
  // the device maximum (less the kernel's static shared memory) once, not to this handle's size
  auto raise_smem = [&](const void* f) -> cudaError_t {
    cudaFuncAttributes fa{};
    cudaError_t e = cudaFuncGetAttributes(&fa, f);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                smem_optin - (int)fa.sharedSizeBytes);
  };
  for (int mode = 0; mode < 3; mode++)
    AES_CK(raise_smem((const void*)pick_plain((int)bits, sgn, mode)));
  for (int mode = 0; mode < 2; mode++)
    AES_CK(raise_smem((const void*)pick_batch((int)bits, sgn, mode)));
  AES_CK(raise_smem((const void*)k_final));
  if (tc_ready) {
    AES_CK(raise_smem((const void*)k_cand_tc<2, false>));
    AES_CK(raise_smem((const void*)k_cand_tc<3, false>));
    AES_CK(raise_smem((const void*)k_cand_tc<2, true>));
    AES_CK(raise_smem((const void*)k_cand_tc<3, true>));
  }
  // the matrix arrays go to the store a view shares; the slow path's key array stays the handle's
  mat_store = std::make_shared<SharedAllocs>();
  mat_store->device = device;
  std::vector<void*> own;
  for (void* q : allocs) (q == (void*)d_allkeys ? own : mat_store->ptrs).push_back(q);
  allocs.swap(own);
  rc = apply_config(c);
  if (rc) return rc;
  AES_CK(cudaDeviceSynchronize());
  return AES_OK;
}

// A view: another handle on base's resident matrix, with its own stream, slow-path key array and
// per-batch buffers (configuration p), so that batches of one matrix run at the same time.
int Engine::build_view(const Engine& b, const aes_params& p) {
  if (p.bits != b.prm.bits || p.quant != b.prm.quant || p.pack_parts != b.prm.pack_parts ||
      p.seed != b.prm.seed || p.device != b.prm.device)
    return fail(AES_ERR_INVALID,
                "bits, quant, pack_parts, seed and device are fixed by the packed matrix");
  prm = p;
  device = b.device;
  AES_CK(cudaSetDevice(device));
  sm_count = b.sm_count;
  smem_optin = b.smem_optin;
  AES_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  AES_CK(cudaEventCreate(&ev0));
  AES_CK(cudaEventCreate(&ev1));
  rows = b.rows; cols = b.cols; bits = b.bits; quant = b.quant; P = b.P;
  nnz = b.nnz; qnnz = b.qnnz; packets = b.packets; tiles = b.tiles; sgn = b.sgn;
  d_tiles = b.d_tiles; d_tile_rowbase = b.d_tile_rowbase; d_rowscale = b.d_rowscale;
  d_tc_ptr = b.d_tc_ptr; d_tc_ent = b.d_tc_ent; tc_nch = b.tc_nch; tc_rtiles = b.tc_rtiles;
  tc_ready = b.tc_ready;
  d_csr_ptr = b.d_csr_ptr; d_csr_col = b.d_csr_col; d_csr_val = b.d_csr_val;
  has_f32 = b.has_f32;
  ld32 = b.ld32; ld8 = b.ld8;
  h_tile_rowbase = b.h_tile_rowbase;
  mat_store = b.mat_store;
  Config c;
  int rc = plan_config(p, &c);
  if (rc) return rc;
  const size_t plan = rows * 4ull + c.plan;
  if (p.mem_limit && plan > p.mem_limit)
    return fail(AES_ERR_NOMEM, "view needs " + std::to_string(plan) +
                                   " device bytes, over the handle limit " +
                                   std::to_string(p.mem_limit));
  size_t freeb = 0, totalb = 0;
  AES_CK(cudaMemGetInfo(&freeb, &totalb));
  if (plan + (64ull << 20) > freeb)
    return fail(AES_ERR_NOMEM, "view needs " + std::to_string(plan) + " device bytes, " +
                                   std::to_string(freeb) + " free");
  if ((rc = dalloc(&d_allkeys, rows)) != AES_OK) return rc;
  rc = apply_config(c);
  if (rc) return rc;
  AES_CK(cudaDeviceSynchronize());
  return AES_OK;
}

// Re-plans CK, split, sample stride, batch tile, k_max, max_batch, flags and the query quantiser
// of a resident matrix without packing it again.  The old buffers are freed first; if the new
// ones cannot be had, the old configuration is restored and the error returned.
int Engine::retune(const aes_params& p) {
  if (p.bits != prm.bits || p.quant != prm.quant || p.pack_parts != prm.pack_parts ||
      p.seed != prm.seed || p.device != prm.device)
    return fail(AES_ERR_INVALID,
                "bits, quant, pack_parts, seed and device are fixed by the packed matrix");
  AES_CK(cudaSetDevice(device));
  Config c;
  int rc = plan_config(p, &c);
  if (rc) return rc;
  if (p.mem_limit && mat_bytes + c.plan > p.mem_limit)
    return fail(AES_ERR_NOMEM, "configuration needs " + std::to_string(mat_bytes + c.plan) +
                                   " device bytes, over the handle limit " +
                                   std::to_string(p.mem_limit));
  AES_CK(cudaDeviceSynchronize());  // runs on caller streams may still read the old buffers
  size_t freeb = 0, totalb = 0;
  AES_CK(cudaMemGetInfo(&freeb, &totalb));
  if (c.plan + (64ull << 20) > freeb + cfg_bytes)
    return fail(AES_ERR_NOMEM, "configuration needs " + std::to_string(c.plan) +
                                   " device bytes, " + std::to_string(freeb + cfg_bytes) +
                                   " available");
  Config old = cur;
  free_config();
  rc = apply_config(c);
  if (rc) {
    std::string why = last_error_cstr();
    free_config();
    if (apply_config(old) != AES_OK) free_config();
    return fail(rc, why);
  }
  AES_CK(cudaDeviceSynchronize());
  return AES_OK;
}

// mode's pass for query q (MODE_SAMPLE: for queries q .. q + nq_y - 1 in one launch)
int Engine::run_plain(int mode, uint32_t q, cudaStream_t s, uint32_t nq_y) {
  PlainArgs a{};
  a.tiles = d_tiles;
  a.tile_rowbase = d_tile_rowbase;
  a.n_tiles = (uint32_t)tiles;
  a.n_rows = rows;
  a.cols = cols;
  a.q8 = d_q8 + (size_t)q * ld8;
  a.rowscale = d_rowscale;
  a.split = split;
  a.slice = slice;
  a.thr = d_thr + (size_t)q * split;
  a.cnt = d_cnt + (size_t)q * split;
  a.surv = d_surv + (size_t)q * split * cap;
  a.cap = cap;
  a.sample_first = d_sample_first;
  a.sample_stride = ss;
  a.n_sample_tiles = n_sample_tiles;
  if (mode == MODE_SAMPLE) a.keys_out = d_sample_keys + (size_t)q * n_sample_rows;
  else if (mode == MODE_ALL) a.keys_out = d_allkeys;
  if (mode != MODE_SAMPLE) nq_y = 1;
  a.q8_ld = (uint32_t)ld8;
  a.keys_ld = (uint32_t)n_sample_rows;
  int grid = plain_grid;
  const int pw = plain_warps((int)bits);
  if (mode == MODE_SAMPLE) {
    // one warp per sample tile for a single query; for several, about two waves of CTAs in all,
    // each warp taking several tiles, so the query table is filled fewer times
    grid = std::min<int>(grid, (int)((n_sample_tiles + pw - 1) / pw));
    if (nq_y > 1) grid = std::min<int>(grid, (int)((2u * (uint32_t)sm_count + nq_y - 1) / nq_y));
  }
  grid = std::max(grid, 1);
  const bool prof = (prm.flags & AES_FLAG_PROFILE) && mode != MODE_SAMPLE;
  int rc = prof ? prof_open(s) : AES_OK;
  if (rc) return rc;
  pick_plain((int)bits, sgn, mode)<<<dim3(grid, nq_y), plain_threads((int)bits), plain_smem, s>>>(a);
  AES_CK(cudaGetLastError());
  if (prof && (rc = prof_close(s))) return rc;
  n_launch++;
  if (mode != MODE_SAMPLE) n_cand++;
  return AES_OK;
}

// The batched pass of mode over every 128-query block of an nq-query batch in one persistent
// launch (blocks walked one after another; each CTA loads a block's query table once)
int Engine::run_batch(int mode, uint32_t nq, cudaStream_t s, uint32_t blk0, uint32_t nblk) {
  BatchArgs a{};
  a.tiles = d_tiles;
  a.tile_rowbase = d_tile_rowbase;
  a.n_tiles = (uint32_t)tiles;
  a.n_rows = rows;
  a.cols = cols;
  a.qtab = d_qtab;
  a.nq = nq;
  a.blk0 = blk0;
  if (!nblk) nblk = (nq + kBatchQ - 1) / kBatchQ - blk0;
  a.rowscale = d_rowscale;
  a.split = split;
  a.slice = slice;
  a.thr = d_thr;
  a.cnt = d_cnt;
  a.surv = d_surv;
  a.cap = cap;
  a.keys_out = d_sample_keys;
  a.sample_first = d_sample_first;
  a.sample_stride = ss;
  a.n_sample_tiles = n_sample_tiles;
  a.n_sample_rows = n_sample_rows;
  int grid = batch_grid;
  if (mode == MODE_SAMPLE)
    grid = std::min<int>(grid, (int)((n_sample_tiles + batch_warps_n - 1) / batch_warps_n));
  grid = std::max(grid, 1);
  const bool prof = (prm.flags & AES_FLAG_PROFILE) && mode != MODE_SAMPLE;
  int rc = prof ? prof_open(s) : AES_OK;
  if (rc) return rc;
  pick_batch((int)bits, sgn, mode)<<<dim3(grid, nblk), batch_warps_n * 32, batch_smem, s>>>(a);
  AES_CK(cudaGetLastError());
  if (prof && (rc = prof_close(s))) return rc;
  n_launch++;
  if (mode != MODE_SAMPLE) n_cand++;
  return AES_OK;
}

int Engine::enqueue(const float* d_q, uint32_t nq, uint32_t k, uint32_t* d_idx, float* d_score,
                    cudaStream_t s, bool pre) {
  AES_CK(cudaMemsetAsync(d_status, 0, nq * 4ull, s));
  if (!pre) {
    k_quantize<<<nq, 256, 0, s>>>(d_q, cols, ld32, (int)bits, (int)quant,
                                  (int)prm.query_quant, d_q8, ld8, d_status);
    AES_CK(cudaGetLastError());
    n_launch++;
  }
  n_launch += 3;  // threshold, select, final
  const bool batched = batch_mode != 1 && (batch_mode != 0 || nq >= 16);
  last_batched = batched;
  const uint32_t nblk = (nq + kBatchQ - 1) / kBatchQ;
  if (batched) {
    k_qtable<<<(uint32_t)((nblk * batch_qtab_words(cols) + 255) / 256), 256, 0, s>>>(
        d_q8, ld8, cols, nq, d_qtab);
    AES_CK(cudaGetLastError());
    n_launch++;
    if (use_tc) {
      for (uint32_t b = 0; b < nblk; b++) {
        const uint32_t nb = std::min<uint32_t>(kBatchQ, nq - b * kBatchQ);
        k_qtable_tc<<<(kTcQ * tc_kpad(cols) + 255) / 256, 256, 0, s>>>(
            d_q8, ld8, cols, b * kTcQ, nb, d_qtab_tc + (size_t)b * tc_qtab_bytes(cols));
        AES_CK(cudaGetLastError());
        n_launch++;
      }
    }
    int rc = run_batch(MODE_SAMPLE, nq, s);
    if (rc) return rc;
  } else {
    for (uint32_t q0 = 0; q0 < nq; q0 += 65535u) {  // every query's sample pass in one launch
      int rc = run_plain(MODE_SAMPLE, q0, s, std::min<uint32_t>(65535u, nq - q0));
      if (rc) return rc;
    }
  }
  if (batched && n_sample_rows) {  // the threshold pass reads each query's keys contiguously
    k_keys_transpose<<<dim3((n_sample_rows + kTransposeRows - 1) / kTransposeRows, nblk), 256, 0, s>>>(
        d_sample_keys, n_sample_rows, nq, d_keys_t);
    AES_CK(cudaGetLastError());
    n_launch++;
  }
  k_threshold<<<dim3(split, nq), kThreadsThr, 0, s>>>(batched ? d_keys_t : d_sample_keys, n_sample_rows, 0,
                                              d_part_sample_begin, split, d_part_r, d_thr, d_cnt);
  AES_CK(cudaGetLastError());
  if (batched) {
    if (use_tc) {
      // two blocks per launch by CTA pairs where there are two; a last odd block alone
      for (uint32_t b = 0; b < nblk;) {
        const bool pair = tc_pair && b + 1 < nblk;
        const uint32_t nb = std::min<uint32_t>((pair ? 2u : 1u) * kBatchQ, nq - b * kBatchQ);
        int rc = run_tc(b, nb, s, pair);
        if (rc) return rc;
        b += pair ? 2u : 1u;
      }
    } else {
      int rc = run_batch(MODE_FILTER, nq, s);
      if (rc) return rc;
    }
  } else {
    for (uint32_t q = 0; q < nq; q++) {
      int rc = run_plain(MODE_FILTER, q, s);
      if (rc) return rc;
    }
  }
  SelectArgs sa{};
  sa.surv = d_surv;
  sa.cnt = d_cnt;
  sa.cap = cap;
  sa.split = split;
  sa.slice = slice;
  sa.n_rows = rows;
  sa.ntop = ntop;
  sa.cand = d_cand;
  sa.cand_key = d_cand_key;
  sa.status = d_status;
  k_select<false><<<dim3(split, nq), 512, 0, s>>>(sa);
  AES_CK(cudaGetLastError());
  FinalArgs fa{};
  fa.csr_ptr = d_csr_ptr;
  fa.csr_col = d_csr_col;
  fa.csr_val = d_csr_val;
  fa.q32 = d_q;
  fa.ld32 = ld32;
  fa.cols = cols;
  fa.cand = d_cand;
  fa.nslots = nslots;
  fa.kp = pow2_at_least(k);
  fa.k = k;
  fa.out_idx = d_idx;
  fa.out_score = d_score;
  fa.status = d_status;
  fa.cand_key = int_final(d_q) ? d_cand_key : nullptr;
  k_final<<<nq, kThreadsFinal, final_smem, s>>>(fa);
  AES_CK(cudaGetLastError());
  return AES_OK;
}

// Replays the launch sequence of enqueue() as one CUDA graph (captured on first use for these
// arguments).  Profiling events are not recorded inside graphs.
int Engine::enqueue_graph(const float* d_q, uint32_t nq, uint32_t k, uint32_t* d_idx,
                          float* d_score, cudaStream_t s, bool pre) {
  GraphKey key{d_q, nq, k, d_idx, d_score, s, pre};
  auto it = graphs.find(key);
  if (it == graphs.end()) {
    if (graphs.size() >= 64) {
      for (auto& g : graphs) cudaGraphExecDestroy(g.second);
      graphs.clear();
    }
    const uint32_t saved_flags = prm.flags;
    prm.flags &= ~AES_FLAG_PROFILE;
    const uint64_t saved_launch = n_launch, saved_cand = n_cand;
    AES_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue(d_q, nq, k, d_idx, d_score, s, pre);
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    prm.flags = saved_flags;
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ce != cudaSuccess) return ::aes::fail(AES_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    cudaGraphExec_t ex = nullptr;
    ce = cudaGraphInstantiate(&ex, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return ::aes::fail(AES_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ce));
    it = graphs.emplace(key, ex).first;
    graph_launches = n_launch - saved_launch;
    graph_cands = n_cand - saved_cand;
    n_launch = saved_launch;
    n_cand = saved_cand;
  }
  AES_CK(cudaGraphLaunch(it->second, s));
  n_launch += graph_launches;
  n_cand += graph_cands;
  n_graph_launch++;
  return AES_OK;
}

// Exact slow path for the queries whose status reports a threshold miss or an overflow: score
// every row, select each partition's Top-CK from the full key array, rescore.
int Engine::repair(uint32_t nq, uint32_t k, uint32_t* d_idx, float* d_score, cudaStream_t s,
                   uint32_t* repaired) {
  AES_CK(cudaMemcpyAsync(h_status, d_status, nq * 4ull, cudaMemcpyDeviceToHost, s));
  AES_CK(cudaStreamSynchronize(s));
  uint32_t nrep = 0;
  for (uint32_t q = 0; q < nq; q++) {
    if (h_status[q] & ST_QUERY) return fail(AES_ERR_QUERY, "query " + std::to_string(q) +
                                               " has negative entries under an unsigned quantiser");
    if (h_status[q] & ST_DEVICE)
      return fail(AES_ERR_CUDA, "tensor-core candidate pass: a bounded wait gave up");
  }
  for (uint32_t q = 0; q < nq; q++) {
    if (!(h_status[q] & (ST_OVERFLOW | ST_MISS))) continue;
    nrep++;
    n_repaired++;
    n_launch += 2;
    int rc = run_plain(MODE_ALL, q, s);
    if (rc) return rc;
    SelectArgs sa{};
    sa.allkeys = d_allkeys;
    sa.q0 = q;
    sa.split = split;
    sa.slice = slice;
    sa.n_rows = rows;
    sa.ntop = ntop;
    sa.cand = d_cand;
    sa.cand_key = d_cand_key;
    sa.status = d_status;
    k_select<true><<<dim3(split, 1), 512, 0, s>>>(sa);
    AES_CK(cudaGetLastError());
    FinalArgs fa{};
    fa.csr_ptr = d_csr_ptr;
    fa.csr_col = d_csr_col;
    fa.csr_val = d_csr_val;
    fa.q32 = last_q32 ? last_q32 + (size_t)q * ld32 : nullptr;
    fa.ld32 = ld32;
    fa.cols = cols;
    fa.cand = d_cand + (size_t)q * nslots;
    fa.nslots = nslots;
    fa.kp = pow2_at_least(k);
    fa.k = k;
    fa.out_idx = d_idx + (size_t)q * k;
    fa.out_score = d_score + (size_t)q * k;
    fa.status = nullptr;
    fa.cand_key = last_int_final ? d_cand_key + (size_t)q * nslots : nullptr;
    k_final<<<1, kThreadsFinal, final_smem, s>>>(fa);
    AES_CK(cudaGetLastError());
  }
  if (nrep) {
    AES_CK(cudaMemsetAsync(d_status, 0, nq * 4ull, s));
    AES_CK(cudaStreamSynchronize(s));
  }
  if (repaired) *repaired = nrep;
  return AES_OK;
}

}  // namespace aes

// =============================================================================================
// C ABI
// =============================================================================================
using aes::Engine;

static const char* const kUnconfigured =
    "the handle has no configuration: a failed aes_retune could not restore the previous one";

struct aes_handle {
  Engine e;
};

extern "C" {

void aes_params_default(aes_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->bits = 6;           // QUANTIZE_B, types.hpp:148
  p->quant = AES_QUANT_SYM_GLOBAL;
  p->query_quant = AES_QQ_NUMPY;
  p->split = 32;         // SPMV_PARTITIONS, types.hpp:39; SPLIT_NUM, search_best_resparse_ratio.py:26
  p->ck = 512;           // APPROXIMATE_K, types.hpp:149
  p->k_max = 100;        // DEFAULT_TOP_K, options.hpp:50
  p->max_batch = 1;
  p->pack_parts = 32;
  p->device = 0;
}

const char* aes_last_error(void) { return aes::last_error_cstr(); }

static int validate_params(const aes_params* p, uint32_t rows, uint32_t cols) {
  using aes::fail;
  if (!p) return fail(AES_ERR_INVALID, "params is NULL");
  if (p->bits != 4 && p->bits != 6 && p->bits != 8)
    return fail(AES_ERR_UNSUPPORTED, "bits must be 4, 6 or 8");
  if (p->quant > AES_QUANT_UNSIGNED_GLOBAL) return fail(AES_ERR_INVALID, "unknown quantiser");
  if (p->query_quant > AES_QQ_TRUNC) return fail(AES_ERR_INVALID, "unknown query quantiser");
  if (p->query_quant == AES_QQ_TRUNC && p->quant != AES_QUANT_SYM_GLOBAL)
    return fail(AES_ERR_INVALID, "the truncating query quantiser is signed");
  if (rows == 0) return fail(AES_ERR_INVALID, "rows must be > 0");
  if (cols == 0 || cols > aes::kMaxCols)
    return fail(AES_ERR_UNSUPPORTED, "cols must be in [1, 1024] (10-bit column field)");
  uint32_t S = p->split <= 1 ? 1 : p->split;
  if (p->ck < S) return fail(AES_ERR_INVALID, "ck must be >= split");
  if (p->ck / S * S > 4096) return fail(AES_ERR_UNSUPPORTED, "ck above 4096");
  if (p->k_max == 0 || p->k_max > 1024) return fail(AES_ERR_UNSUPPORTED, "k_max must be in [1, 1024]");
  if (p->max_batch == 0 || p->max_batch > 65535) return fail(AES_ERR_INVALID, "max_batch out of range");
  if (p->batch_warps > 32) return fail(AES_ERR_INVALID, "batch_warps above 32");
  return AES_OK;
}

static int create_common(aes::HostCSR& m, const aes_params* p, aes_handle** out) {
  aes_handle* h = new (std::nothrow) aes_handle();
  if (!h) return aes::fail(AES_ERR_NOMEM, "host allocation failed");
  int rc = h->e.build(m, *p);
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return AES_OK;
}

int aes_create(const uint32_t* row, const uint32_t* col, const float* val, uint32_t rows,
               uint32_t cols, uint64_t nnz, const aes_params* p, aes_handle** out) {
  if (!out) return aes::fail(AES_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate_params(p, rows, cols);
  if (rc) return rc;
  if (nnz && (!row || !col || !val)) return aes::fail(AES_ERR_INVALID, "NULL COO array");
  aes::HostCSR m;
  rc = aes::coo_to_csr(row, col, val, rows, cols, nnz, &m);
  if (rc) return rc;
  return create_common(m, p, out);
}

int aes_create_csr(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                   uint32_t cols, const aes_params* p, aes_handle** out) {
  if (!out) return aes::fail(AES_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate_params(p, rows, cols);
  if (rc) return rc;
  if (!ptr) return aes::fail(AES_ERR_INVALID, "NULL CSR array");
  if (ptr[rows] && (!col || !val)) return aes::fail(AES_ERR_INVALID, "NULL CSR array");
  rc = aes::check_csr(ptr, col, rows, cols);
  if (rc) return rc;
  aes::HostCSR m;
  m.rows = rows;
  m.cols = cols;
  m.ptr.assign(ptr, ptr + rows + 1);
  m.col.assign(col, col + ptr[rows]);
  m.val.assign(val, val + ptr[rows]);
  return create_common(m, p, out);
}

int aes_create_quantized(const uint32_t* row, const uint32_t* col, const int8_t* q_val,
                         const float* val, uint32_t rows, uint32_t cols, uint64_t nnz,
                         const aes_params* p, aes_handle** out) {
  if (!out) return aes::fail(AES_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate_params(p, rows, cols);
  if (rc) return rc;
  if (p->quant != AES_QUANT_SYM_GLOBAL)
    return aes::fail(AES_ERR_UNSUPPORTED, "pre-quantised matrices take the symmetric B-bit values");
  if (nnz && (!row || !col || !q_val)) return aes::fail(AES_ERR_INVALID, "NULL COO array");
  aes::HostCSR m;
  rc = aes::coo_to_csr(row, col, val, rows, cols, nnz, &m, q_val);
  if (rc) return rc;
  m.prequantized = true;
  if (!val) m.val.clear();
  return create_common(m, p, out);
}

int aes_pack_host(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                  uint32_t cols, const aes_params* p, uint8_t* packets, uint64_t cap_packets,
                  uint64_t* n_packets, uint32_t* tile_rowbase) {
  if (!n_packets || !ptr) return aes::fail(AES_ERR_INVALID, "NULL argument");
  int rc = validate_params(p, rows, cols);
  if (rc) return rc;
  rc = aes::check_csr(ptr, col, rows, cols);
  if (rc) return rc;
  aes::HostCSR m;
  m.rows = rows;
  m.cols = cols;
  m.ptr.assign(ptr, ptr + rows + 1);
  m.col.assign(col, col + ptr[rows]);
  m.val.assign(val, val + ptr[rows]);
  aes::PackedMatrix pm;
  rc = aes::quantize_and_pack(m, *p, &pm);
  if (rc) return rc;
  *n_packets = pm.packets;
  if (packets) {
    if (cap_packets < pm.packets) return aes::fail(AES_ERR_INVALID, "packet buffer too small");
    std::vector<uint8_t> flat;
    aes::untile_packets(pm, &flat);
    std::memcpy(packets, flat.data(), flat.size());
  }
  if (tile_rowbase) std::memcpy(tile_rowbase, pm.tile_rowbase.data(), pm.tile_rowbase.size() * 4);
  return AES_OK;
}

int aes_pack_tc_host(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                     uint32_t cols, const aes_params* p, uint32_t* tile_ptr, uint64_t cap_ptr,
                     uint32_t* entries, uint64_t cap_entries, uint64_t* n_ptr,
                     uint64_t* n_entries) {
  if (!n_ptr || !n_entries || !ptr) return aes::fail(AES_ERR_INVALID, "NULL argument");
  int rc = validate_params(p, rows, cols);
  if (rc) return rc;
  rc = aes::check_csr(ptr, col, rows, cols);
  if (rc) return rc;
  aes::HostCSR m;
  m.rows = rows;
  m.cols = cols;
  m.ptr.assign(ptr, ptr + rows + 1);
  m.col.assign(col, col + ptr[rows]);
  m.val.assign(val, val + ptr[rows]);
  aes::PackedMatrix pm;
  rc = aes::quantize_and_pack(m, *p, &pm);
  if (rc) return rc;
  *n_ptr = pm.tc_ptr.size();
  *n_entries = pm.tc_ent.size();
  if (tile_ptr) {
    if (cap_ptr < pm.tc_ptr.size()) return aes::fail(AES_ERR_INVALID, "tile_ptr buffer too small");
    std::memcpy(tile_ptr, pm.tc_ptr.data(), pm.tc_ptr.size() * 4);
  }
  if (entries) {
    if (cap_entries < pm.tc_ent.size()) return aes::fail(AES_ERR_INVALID, "entry buffer too small");
    std::memcpy(entries, pm.tc_ent.data(), pm.tc_ent.size() * 4);
  }
  return AES_OK;
}

int aes_create_view(const aes_handle* base, const aes_params* p, aes_handle** out) {
  if (!base || !out) return aes::fail(AES_ERR_INVALID, "NULL argument");
  *out = nullptr;
  const aes_params prm = p ? *p : base->e.prm;
  int rc = validate_params(&prm, base->e.rows, base->e.cols);
  if (rc) return rc;
  if (!base->e.mat_store) return aes::fail(AES_ERR_STATE, "the base handle holds no matrix");
  aes_handle* h = new (std::nothrow) aes_handle();
  if (!h) return aes::fail(AES_ERR_NOMEM, "host allocation failed");
  rc = h->e.build_view(base->e, prm);
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return AES_OK;
}

int aes_destroy(aes_handle* h) {
  if (!h) return AES_OK;
  delete h;
  return AES_OK;
}

int aes_retune(aes_handle* h, const aes_params* p) {
  if (!h) return aes::fail(AES_ERR_INVALID, "NULL handle");
  int rc = validate_params(p, h->e.rows, h->e.cols);
  if (rc) return rc;
  return h->e.retune(*p);
}

int aes_get_info(const aes_handle* h, aes_info* info) {
  if (!h || !info) return aes::fail(AES_ERR_INVALID, "NULL argument");
  const Engine& e = h->e;
  std::memset(info, 0, sizeof(*info));
  info->rows = e.rows;
  info->cols = e.cols;
  info->bits = e.bits;
  info->packet_elems = e.P;
  info->nnz = e.nnz;
  info->quantized_nnz = e.qnnz;
  info->packets = e.packets;
  info->tiles = e.tiles;
  info->packet_bytes = e.packets * 64ull;
  info->device_bytes = e.bytes;
  info->split = e.split;
  info->ck = e.nslots;
  info->ck_effective = e.ck_eff;
  info->sample_tiles = e.n_sample_tiles;
  info->sample_rows = e.n_sample_rows;
  info->max_batch = e.maxB;
  info->batch_tile = e.batch_mode == 1 ? 1 : aes::dev::kBatchQ;
  info->tensor_tiles = e.use_tc ? 1u : 0u;
  info->exact_pass = e.has_f32 ? 1u : 0u;
  info->batch_warps = e.batch_mode == 1 ? 0u : (uint32_t)e.batch_warps_n;
  return AES_OK;
}

int aes_set_query(aes_handle* h, const float* q, uint32_t nq) {
  if (!h || !q) return aes::fail(AES_ERR_INVALID, "NULL argument");
  Engine& e = h->e;
  if (!e.configured) return aes::fail(AES_ERR_STATE, kUnconfigured);
  if (nq == 0 || nq > e.maxB) return aes::fail(AES_ERR_INVALID, "nq must be in [1, max_batch]");
  cudaSetDevice(e.device);
  for (uint32_t i = 0; i < nq; i++) std::memcpy(e.h_q32 + (size_t)i * e.ld32, q + (size_t)i * e.cols, e.cols * 4ull);
  AES_CK(cudaMemcpyAsync(e.d_q32, e.h_q32, (size_t)nq * e.ld32 * 4, cudaMemcpyHostToDevice, e.stream));
  e.nq_loaded = nq;
  e.q_pre = false;
  e.q32_given = true;
  return AES_OK;
}

int aes_set_query_quantized(aes_handle* h, const int8_t* q, const float* q_f32, uint32_t nq) {
  if (!h || !q) return aes::fail(AES_ERR_INVALID, "NULL argument");
  Engine& e = h->e;
  if (!e.configured) return aes::fail(AES_ERR_STATE, kUnconfigured);
  if (nq == 0 || nq > e.maxB) return aes::fail(AES_ERR_INVALID, "nq must be in [1, max_batch]");
  if (e.quant != AES_QUANT_SYM_GLOBAL)
    return aes::fail(AES_ERR_UNSUPPORTED, "pre-quantised queries take the symmetric B-bit values");
  const int lo = -(1 << (e.bits - 1)), hi = (1 << (e.bits - 1)) - 1;
  for (uint32_t i = 0; i < nq; i++) {
    for (uint32_t c = 0; c < e.cols; c++) {
      const int v = q[(size_t)i * e.cols + c];
      if (v < lo || v > hi) return aes::fail(AES_ERR_QUERY, "query value outside the signed B-bit range");
    }
  }
  cudaSetDevice(e.device);
  std::memset(e.h_q8, 0, (size_t)nq * e.ld8);
  for (uint32_t i = 0; i < nq; i++) std::memcpy(e.h_q8 + (size_t)i * e.ld8, q + (size_t)i * e.cols, e.cols);
  AES_CK(cudaMemcpyAsync(e.d_q8, e.h_q8, (size_t)nq * e.ld8, cudaMemcpyHostToDevice, e.stream));
  if (q_f32) {
    for (uint32_t i = 0; i < nq; i++)
      std::memcpy(e.h_q32 + (size_t)i * e.ld32, q_f32 + (size_t)i * e.cols, e.cols * 4ull);
    AES_CK(cudaMemcpyAsync(e.d_q32, e.h_q32, (size_t)nq * e.ld32 * 4, cudaMemcpyHostToDevice, e.stream));
  }
  e.nq_loaded = nq;
  e.q_pre = true;
  e.q32_given = q_f32 != nullptr;
  return AES_OK;
}

int aes_run(aes_handle* h, uint32_t k, uint32_t* out_idx, float* out_score, uint64_t* ns) {
  if (!h || !out_idx || !out_score) return aes::fail(AES_ERR_INVALID, "NULL argument");
  Engine& e = h->e;
  if (!e.nq_loaded) return aes::fail(AES_ERR_STATE, "aes_set_query must come first");
  if (k == 0 || k > e.prm.k_max) return aes::fail(AES_ERR_INVALID, "k must be in [1, k_max]");
  cudaSetDevice(e.device);
  const uint32_t nq = e.nq_loaded;
  const float* dq = e.q32_given ? e.d_q32 : nullptr;
  e.last_q32 = dq;
  e.last_int_final = e.int_final(dq);
  AES_CK(cudaEventRecord(e.ev0, e.stream));
  int rc = (e.prm.flags & AES_FLAG_GRAPHS)
               ? e.enqueue_graph(dq, nq, k, e.d_out_idx, e.d_out_score, e.stream, e.q_pre)
               : e.enqueue(dq, nq, k, e.d_out_idx, e.d_out_score, e.stream, e.q_pre);
  if (rc) return rc;
  AES_CK(cudaEventRecord(e.ev1, e.stream));
  uint32_t rep = 0;
  rc = e.repair(nq, k, e.d_out_idx, e.d_out_score, e.stream, &rep);
  if (rc) return rc;
  AES_CK(cudaMemcpyAsync(out_idx, e.d_out_idx, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, e.stream));
  AES_CK(cudaMemcpyAsync(out_score, e.d_out_score, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, e.stream));
  AES_CK(cudaStreamSynchronize(e.stream));
  if (ns) {
    float ms = 0.0f;
    AES_CK(cudaEventElapsedTime(&ms, e.ev0, e.ev1));
    *ns = (uint64_t)((double)ms * 1e6);
  }
  e.last_nq = nq;
  e.last_k = k;
  e.ran = true;
  return AES_OK;
}

int aes_run_device(aes_handle* h, const float* d_queries, uint32_t nq, uint32_t k,
                   uint32_t* d_idx, float* d_score, void* stream) {
  if (!h || !d_queries || !d_idx || !d_score) return aes::fail(AES_ERR_INVALID, "NULL argument");
  Engine& e = h->e;
  if (!e.configured) return aes::fail(AES_ERR_STATE, kUnconfigured);
  if (nq == 0 || nq > e.maxB) return aes::fail(AES_ERR_INVALID, "nq must be in [1, max_batch]");
  if (k == 0 || k > e.prm.k_max) return aes::fail(AES_ERR_INVALID, "k must be in [1, k_max]");
  cudaSetDevice(e.device);
  cudaStream_t s = stream ? (cudaStream_t)stream : e.stream;
  if (e.ld32 != e.cols) {
    // the device kernels read queries with the padded stride; stage through the handle buffer
    AES_CK(cudaMemcpy2DAsync(e.d_q32, e.ld32 * 4ull, d_queries, e.cols * 4ull, e.cols * 4ull, nq,
                             cudaMemcpyDeviceToDevice, s));
    d_queries = e.d_q32;
  }
  e.last_q32 = d_queries;
  e.last_int_final = e.int_final(d_queries);
  int rc = (e.prm.flags & AES_FLAG_GRAPHS) ? e.enqueue_graph(d_queries, nq, k, d_idx, d_score, s)
                                           : e.enqueue(d_queries, nq, k, d_idx, d_score, s);
  if (rc) return rc;
  e.last_nq = nq;
  e.last_k = k;
  e.last_idx = d_idx;
  e.last_score = d_score;
  e.last_stream = s;
  e.last_from_device = true;
  e.ran = true;
  return AES_OK;
}

int aes_finish(aes_handle* h, uint32_t* repaired) {
  if (!h) return aes::fail(AES_ERR_INVALID, "NULL handle");
  Engine& e = h->e;
  if (repaired) *repaired = 0;
  if (!e.last_from_device) return AES_OK;
  cudaSetDevice(e.device);
  int rc = e.repair(e.last_nq, e.last_k, e.last_idx, e.last_score, e.last_stream, repaired);
  e.last_from_device = false;
  return rc;
}

int aes_get_stats(aes_handle* h, aes_stats* st, int reset) {
  if (!h || !st) return aes::fail(AES_ERR_INVALID, "NULL argument");
  Engine& e = h->e;
  cudaSetDevice(e.device);
  int rc = e.collect_profile();
  if (rc) return rc;
  st->launches = e.n_launch;
  st->cand_launches = e.n_cand;
  st->cand_ms = e.prof_ms;
  st->cand_timed = e.prof_n;
  st->repaired = e.n_repaired;
  if (reset) {
    e.n_launch = e.n_cand = e.n_repaired = e.prof_n = 0;
    e.prof_ms = 0.0;
  }
  return AES_OK;
}

int aes_run_exact(aes_handle* h, uint32_t k, uint32_t* out_idx, float* out_score, uint64_t* ns) {
  using namespace aes::dev;
  if (!h || !out_idx || !out_score) return aes::fail(AES_ERR_INVALID, "NULL argument");
  Engine& e = h->e;
  if (!e.nq_loaded) return aes::fail(AES_ERR_STATE, "aes_set_query must come first");
  if (k == 0 || k > e.prm.k_max) return aes::fail(AES_ERR_INVALID, "k must be in [1, k_max]");
  if (!e.has_f32) return aes::fail(AES_ERR_STATE, "the matrix was created without FP32 values");
  if (!e.q32_given) return aes::fail(AES_ERR_STATE, "the loaded queries have no FP32 values");
  AES_CK(cudaSetDevice(e.device));
  uint32_t kp = 1;
  while (kp < k) kp <<= 1;
  // Filtered select: every S-th row key is a sample; its r-th largest key lies below the K-th
  // largest key of all rows except with probability 1e-12 (binomial tail), so only the rows at or
  // above it need the select.  S is the largest power of two whose expected survivors fit the
  // survivor buffer; a miss or an overflow is detected by the select and falls back to the
  // select over every row, so the result is exact either way.
  uint32_t S = 0, r = 0;
  for (uint32_t cs = 1024; cs >= 2 && e.rows >= 4u * k; cs >>= 1) {
    const uint32_t nsm = (e.rows + cs - 1) / cs;
    const double f = 1.0 / cs;
    const uint32_t n1 = k - 1;
    uint32_t rr = (uint32_t)std::floor(n1 * f);
    while (rr <= n1 && aes::binom_tail(n1, f, rr) > 1e-12) rr++;
    rr = std::max<uint32_t>(rr, 1);
    if (rr > nsm) continue;
    if (2.0 * rr / f + k + 64.0 <= (double)e.cap) {
      S = cs;
      r = rr;
      break;
    }
  }
  if (S) {
    const uint32_t aux[3] = {0u, (e.rows + S - 1) / S, r};
    AES_CK(cudaMemcpy(e.d_exact_aux, aux, sizeof(aux), cudaMemcpyHostToDevice));
  }
  FinalArgs fa{};
  fa.csr_ptr = e.d_csr_ptr;
  fa.csr_col = e.d_csr_col;
  fa.csr_val = e.d_csr_val;
  fa.ld32 = e.ld32;
  fa.cols = e.cols;
  fa.cand = e.d_exact_cand;
  fa.nslots = k;
  fa.kp = kp;
  fa.k = k;
  fa.out_idx = e.d_out_idx;
  fa.out_score = e.d_out_score;
  fa.status = nullptr;
  fa.cand_key = nullptr;
  SelectArgs sa{};
  sa.q0 = 0;
  sa.split = 1;
  sa.slice = e.rows;
  sa.n_rows = e.rows;
  sa.ntop = k;
  sa.cand = e.d_exact_cand;
  sa.cand_key = e.d_exact_key;
  sa.status = e.d_status;
  float total_ms = 0.0f;
  for (uint32_t q = 0; q < e.nq_loaded; q++) {
    fa.q32 = e.d_q32 + (size_t)q * e.ld32;
    AES_CK(cudaMemsetAsync(e.d_status, 0, 4, e.stream));
    AES_CK(cudaEventRecord(e.ev0, e.stream));
    k_exact_all<<<e.sm_count * 8, kExactWarps * 32, exact_all_smem_bytes(e.cols), e.stream>>>(
        e.d_csr_ptr, e.d_csr_col, e.d_csr_val, e.d_q32 + (size_t)q * e.ld32, e.cols, e.rows,
        e.d_allkeys);
    AES_CK(cudaGetLastError());
    if (S) {
      k_threshold<<<dim3(1, 1), kThreadsThr, 0, e.stream>>>(e.d_allkeys, 0, S, e.d_exact_aux, 1,
                                                           e.d_exact_aux + 2, e.d_thr, e.d_cnt);
      AES_CK(cudaGetLastError());
      k_filter_keys<<<e.sm_count * 4, 256, 0, e.stream>>>(e.d_allkeys, e.rows, e.d_thr, e.d_cnt,
                                                         e.d_surv, e.cap);
      AES_CK(cudaGetLastError());
      sa.surv = e.d_surv;
      sa.cnt = e.d_cnt;
      sa.cap = e.cap;
      k_select<false><<<dim3(1, 1), 512, 0, e.stream>>>(sa);
    } else {
      sa.allkeys = e.d_allkeys;
      k_select<true><<<dim3(1, 1), 512, 0, e.stream>>>(sa);
    }
    AES_CK(cudaGetLastError());
    k_final<<<1, kThreadsFinal, e.final_smem, e.stream>>>(fa);
    AES_CK(cudaGetLastError());
    AES_CK(cudaEventRecord(e.ev1, e.stream));
    AES_CK(cudaMemcpyAsync(e.h_status, e.d_status, 4, cudaMemcpyDeviceToHost, e.stream));
    AES_CK(cudaStreamSynchronize(e.stream));
    float ms = 0.0f;
    AES_CK(cudaEventElapsedTime(&ms, e.ev0, e.ev1));
    total_ms += ms;
    if (S && e.h_status[0]) {  // the sample bound missed or the buffer overflowed: every row
      AES_CK(cudaEventRecord(e.ev0, e.stream));
      sa.allkeys = e.d_allkeys;
      k_select<true><<<dim3(1, 1), 512, 0, e.stream>>>(sa);
      AES_CK(cudaGetLastError());
      k_final<<<1, kThreadsFinal, e.final_smem, e.stream>>>(fa);
      AES_CK(cudaGetLastError());
      AES_CK(cudaEventRecord(e.ev1, e.stream));
      AES_CK(cudaStreamSynchronize(e.stream));
      AES_CK(cudaEventElapsedTime(&ms, e.ev0, e.ev1));
      total_ms += ms;
      e.n_repaired++;
    }
    AES_CK(cudaMemcpyAsync(out_idx + (size_t)q * k, e.d_out_idx, k * 4ull, cudaMemcpyDeviceToHost, e.stream));
    AES_CK(cudaMemcpyAsync(out_score + (size_t)q * k, e.d_out_score, k * 4ull, cudaMemcpyDeviceToHost, e.stream));
    AES_CK(cudaStreamSynchronize(e.stream));
  }
  if (ns) *ns = (uint64_t)((double)total_ms * 1e6);
  return AES_OK;
}

int aes_score_all(aes_handle* h, const float* q, uint32_t* keys) {
  if (!h || !q || !keys) return aes::fail(AES_ERR_INVALID, "NULL argument");
  Engine& e = h->e;
  if (!e.configured) return aes::fail(AES_ERR_STATE, kUnconfigured);
  cudaSetDevice(e.device);
  std::memcpy(e.h_q32, q, e.cols * 4ull);
  AES_CK(cudaMemcpyAsync(e.d_q32, e.h_q32, e.ld32 * 4ull, cudaMemcpyHostToDevice, e.stream));
  AES_CK(cudaMemsetAsync(e.d_status, 0, 4, e.stream));
  aes::dev::k_quantize<<<1, 256, 0, e.stream>>>(e.d_q32, e.cols, e.ld32, (int)e.bits, (int)e.quant,
                                                (int)e.prm.query_quant, e.d_q8, e.ld8, e.d_status);
  AES_CK(cudaGetLastError());
  int rc = e.run_plain(aes::dev::MODE_ALL, 0, e.stream);
  if (rc) return rc;
  uint32_t st = 0;
  AES_CK(cudaMemcpyAsync(keys, e.d_allkeys, e.rows * 4ull, cudaMemcpyDeviceToHost, e.stream));
  AES_CK(cudaMemcpyAsync(&st, e.d_status, 4, cudaMemcpyDeviceToHost, e.stream));
  AES_CK(cudaStreamSynchronize(e.stream));
  e.nq_loaded = 0;
  if (st & aes::dev::ST_QUERY) return aes::fail(AES_ERR_QUERY, "query has negative entries under an unsigned quantiser");
  return AES_OK;
}

int aes_read_candidates(aes_handle* h, uint32_t query, uint32_t* idx, int32_t* score_i32,
                        float* key_f32, uint32_t cap, uint32_t* n) {
  if (!h || !n) return aes::fail(AES_ERR_INVALID, "NULL argument");
  Engine& e = h->e;
  if (!e.ran) return aes::fail(AES_ERR_STATE, "no run yet");
  if (query >= e.last_nq) return aes::fail(AES_ERR_INVALID, "query index out of range");
  cudaSetDevice(e.device);
  std::vector<uint32_t> rows(e.nslots), keys(e.nslots);
  AES_CK(cudaMemcpy(rows.data(), e.d_cand + (size_t)query * e.nslots, e.nslots * 4ull, cudaMemcpyDeviceToHost));
  AES_CK(cudaMemcpy(keys.data(), e.d_cand_key + (size_t)query * e.nslots, e.nslots * 4ull, cudaMemcpyDeviceToHost));
  std::vector<std::pair<uint32_t, uint32_t>> c;
  // AES_FLAG_POSITIVE: Q_read_result's filter (host_spmv_ucsr.cpp:709) keeps scores above 0
  // only; the integer key of score s is s ^ 2^31 and the FP32 key of x > 0 is above 2^31 as well
  const bool positive = (e.prm.flags & AES_FLAG_POSITIVE) != 0;
  for (uint32_t i = 0; i < e.nslots; i++)
    if (rows[i] != 0xFFFFFFFFu && (!positive || keys[i] > 0x80000000u)) c.emplace_back(keys[i], rows[i]);
  std::sort(c.begin(), c.end(), [](const std::pair<uint32_t, uint32_t>& a,
                                   const std::pair<uint32_t, uint32_t>& b) {
    return a.first != b.first ? a.first > b.first : a.second > b.second;
  });
  uint32_t m = (uint32_t)std::min<size_t>(c.size(), cap);
  for (uint32_t i = 0; i < m; i++) {
    if (idx) idx[i] = c[i].second;
    uint32_t kk = c[i].first;
    bool fkey = (e.quant == AES_QUANT_UNSIGNED_ROW);
    float kf;
    if (fkey) {
      uint32_t u = (kk & 0x80000000u) ? (kk & 0x7FFFFFFFu) : ~kk;
      std::memcpy(&kf, &u, 4);
    } else {
      kf = (float)(int32_t)(kk ^ 0x80000000u);
    }
    if (key_f32) key_f32[i] = kf;
    if (score_i32) score_i32[i] = fkey ? 0 : (int32_t)(kk ^ 0x80000000u);
  }
  *n = (uint32_t)c.size();
  return AES_OK;
}

}  // extern "C"

// =============================================================================================
// No-allocation entry point
// =============================================================================================
// Per-query scratch of aes_run_noalloc lives in this fixed device array instead of memory the
// call allocates.  The array is part of the library's device image: every GPU that loads the
// library holds these bytes until the process exits.
static constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[256] = {};  // device address of g_noalloc_scratch, per device ordinal

// Device address of the scratch array on the current device (looked up once per device; host
// code must not use the symbol itself as an address).
int noalloc_scratch(int dev, unsigned char** out) {
  if (dev < 0 || dev >= 256) return aes::fail(AES_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return aes::fail(AES_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_ptr[dev]);
  return AES_OK;
}

struct NoAllocLayout {
  size_t q8, skeys, thr, cnt, surv, cand, cand_key, status, total;
};

NoAllocLayout noalloc_layout(const aes::Engine& e) {
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  NoAllocLayout L{};
  size_t o = 0;
  L.q8 = o;       o += up(e.ld8);
  L.skeys = o;    o += up((size_t)std::max<uint32_t>(e.n_sample_rows, 1) * 4);
  L.thr = o;      o += up((size_t)e.split * 4);
  L.cnt = o;      o += up((size_t)e.split * 4);
  L.surv = o;     o += up((size_t)e.split * e.cap * 8);
  L.cand = o;     o += up((size_t)std::max<uint32_t>(e.nslots, 1) * 4);
  L.cand_key = o; o += up((size_t)std::max<uint32_t>(e.nslots, 1) * 4);
  L.status = o;   o += 256;
  L.total = o;
  return L;
}

}  // namespace

extern "C" int aes_run_noalloc(aes_handle* h, const float* d_query, uint32_t k, uint32_t* d_idx,
                               float* d_score, void* stream) {
  using namespace aes::dev;
  if (!h || !d_query || !d_idx || !d_score) return aes::fail(AES_ERR_INVALID, "NULL argument");
  aes::Engine& e = h->e;
  if (!e.configured) return aes::fail(AES_ERR_STATE, kUnconfigured);
  if (k == 0 || k > e.prm.k_max) return aes::fail(AES_ERR_INVALID, "k must be in [1, k_max]");
  AES_CK(cudaSetDevice(e.device));
  const NoAllocLayout L = noalloc_layout(e);
  if (L.total > kNoAllocScratchBytes)
    return aes::fail(AES_ERR_UNSUPPORTED,
                     "aes_run_noalloc: this matrix needs " + std::to_string(L.total) +
                         " bytes of per-query scratch, over the fixed " +
                         std::to_string(kNoAllocScratchBytes) + "-byte limit");
  unsigned char* base = nullptr;
  int rc = noalloc_scratch(e.device, &base);
  if (rc) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : e.stream;
  int8_t* q8 = reinterpret_cast<int8_t*>(base + L.q8);
  uint32_t* skeys = reinterpret_cast<uint32_t*>(base + L.skeys);
  uint32_t* thr = reinterpret_cast<uint32_t*>(base + L.thr);
  uint32_t* cnt = reinterpret_cast<uint32_t*>(base + L.cnt);
  uint2* surv = reinterpret_cast<uint2*>(base + L.surv);
  uint32_t* cand = reinterpret_cast<uint32_t*>(base + L.cand);
  uint32_t* cand_key = reinterpret_cast<uint32_t*>(base + L.cand_key);
  uint32_t* status = reinterpret_cast<uint32_t*>(base + L.status);

  // the array keeps the previous call's contents: the status word starts at zero, the survivor
  // counters are zeroed by k_threshold, every other region is fully written before it is read
  AES_CK(cudaMemsetAsync(status, 0, 4, s));
  k_quantize<<<1, 256, 0, s>>>(d_query, e.cols, e.ld32, (int)e.bits, (int)e.quant,
                               (int)e.prm.query_quant, q8, e.ld8, status);
  AES_CK(cudaGetLastError());
  auto plain = [&](int mode, uint32_t* keys_out) -> int {
    PlainArgs a{};
    a.tiles = e.d_tiles;
    a.tile_rowbase = e.d_tile_rowbase;
    a.n_tiles = (uint32_t)e.tiles;
    a.n_rows = e.rows;
    a.cols = e.cols;
    a.q8 = q8;
    a.rowscale = e.d_rowscale;
    a.split = e.split;
    a.slice = e.slice;
    a.thr = thr;
    a.cnt = cnt;
    a.surv = surv;
    a.cap = e.cap;
    a.keys_out = keys_out;
    a.sample_first = e.d_sample_first;
    a.sample_stride = e.ss;
    a.n_sample_tiles = e.n_sample_tiles;
    int grid = e.plain_grid;
    if (mode == MODE_SAMPLE)
      grid = std::min<int>(grid, (int)((e.n_sample_tiles + plain_warps((int)e.bits) - 1) /
                                       plain_warps((int)e.bits)));
    grid = std::max(grid, 1);
    aes::pick_plain((int)e.bits, e.sgn, mode)<<<grid, plain_threads((int)e.bits), e.plain_smem, s>>>(a);
    AES_CK(cudaGetLastError());
    return AES_OK;
  };
  if ((rc = plain(MODE_SAMPLE, skeys))) return rc;
  k_threshold<<<dim3(e.split, 1), kThreadsThr, 0, s>>>(skeys, e.n_sample_rows, 0, e.d_part_sample_begin,
                                               e.split, e.d_part_r, thr, cnt);
  AES_CK(cudaGetLastError());
  if ((rc = plain(MODE_FILTER, nullptr))) return rc;
  SelectArgs sa{};
  sa.surv = surv;
  sa.cnt = cnt;
  sa.cap = e.cap;
  sa.split = e.split;
  sa.slice = e.slice;
  sa.n_rows = e.rows;
  sa.ntop = e.ntop;
  sa.cand = cand;
  sa.cand_key = cand_key;
  sa.status = status;
  k_select<false><<<dim3(e.split, 1), 512, 0, s>>>(sa);
  AES_CK(cudaGetLastError());
  FinalArgs fa{};
  fa.csr_ptr = e.d_csr_ptr;
  fa.csr_col = e.d_csr_col;
  fa.csr_val = e.d_csr_val;
  fa.q32 = d_query;
  fa.ld32 = e.ld32;
  fa.cols = e.cols;
  fa.cand = cand;
  fa.nslots = e.nslots;
  fa.kp = aes::pow2_at_least(k);
  fa.k = k;
  fa.out_idx = d_idx;
  fa.out_score = d_score;
  fa.status = status;
  fa.cand_key = e.has_f32 ? nullptr : cand_key;
  k_final<<<1, kThreadsFinal, e.final_smem, s>>>(fa);
  AES_CK(cudaGetLastError());
  // counted like aes_run_device's launches: quantise, sample pass, threshold, filter pass,
  // select, final
  e.n_launch += 6;
  e.n_cand += 1;
  uint32_t st = 0;
  AES_CK(cudaMemcpyAsync(&st, status, 4, cudaMemcpyDeviceToHost, s));
  AES_CK(cudaStreamSynchronize(s));
  if (st & ST_QUERY) return aes::fail(AES_ERR_QUERY, "query has negative entries under an unsigned quantiser");
  if (st & (ST_MISS | ST_OVERFLOW)) {
    e.n_launch += 3;
    e.n_cand += 1;
    e.n_repaired += 1;
    // exact slow path: every row's key into the handle's key array (reserved at creation),
    // each partition's Top-CK from it, then the FP32 rescoring
    if ((rc = plain(MODE_ALL, e.d_allkeys))) return rc;
    sa.allkeys = e.d_allkeys;
    sa.q0 = 0;
    k_select<true><<<dim3(e.split, 1), 512, 0, s>>>(sa);
    AES_CK(cudaGetLastError());
    fa.status = nullptr;
    k_final<<<1, kThreadsFinal, e.final_smem, s>>>(fa);
    AES_CK(cudaGetLastError());
    AES_CK(cudaStreamSynchronize(s));
  }
  return AES_OK;
}
