// aes_select.cuh -- the stages after the candidate pass of the two-stage Top-K SpMV engine, and
// the query quantiser before it (reference: zhaijiaqi/AccelES):
//   k_quantize        quantify_vector (quantify_util.py:31-49) / quantize_vec
//                     (quantize_utils.hpp:8-18): float64 results in integer arithmetic, one CTA per query
//   k_threshold       per (query, partition) lower bound of the Top-CK boundary from a sample
//   k_select          exact Top-CK per partition, (key desc, row desc)
//                     (split_approximate, quantify_util.py:173-196; sort_tuples order)
//   k_final           FP32 rescoring of the candidates (quantify_util.py:354-356 in FP32;
//                     gold_algorithms.hpp:211-239 summation order) and the final Top-K
//   k_exact_all, k_filter_keys   the FP32-only Top-K of every row
#pragma once

#include "aes_kernels.cuh"

namespace aes {
namespace dev {

// ---------------------------------------------------------------------------------------------
// query quantiser: one CTA per query.  The integer query is bit-identical to quantify_vector
// (quantify_util.py:31-49) applied to the float64 upcast of the FP32 query: numpy's binary64
// division and multiplication (round to nearest even) and round-half-to-even are reproduced in
// integer arithmetic (aes_qexact.hpp), so no FP64 runs on the GPU.
// quant: 0 symmetric, 1/2 unsigned (per query); qq: 0 numpy, 1 quantize_vec truncation.
// ---------------------------------------------------------------------------------------------
__global__ void k_quantize(const float* __restrict__ q32, uint32_t cols, uint32_t ld32, int bits,
                           int quant, int qq, int8_t* __restrict__ q8, uint32_t ld8,
                           uint32_t* __restrict__ status) {
  __shared__ float red[32];
  __shared__ int negs;
  const float* x = q32 + (size_t)blockIdx.x * ld32;
  int8_t* o = q8 + (size_t)blockIdx.x * ld8;
  if (qq == 1) {  // quantize_utils.hpp:8-18 (ap_fixed<32,B,AP_TRN_ZERO>, to_int, ap_int<B>)
    const int F = 32 - bits;
    for (uint32_t j = threadIdx.x; j < cols; j += blockDim.x) {
      const int32_t X32 = qx::trunc_scaled30(x[j]);  // x * 2^(B-2+F), truncated, 32-bit wrap
      int32_t n = X32 / (int32_t)(1u << F);
      int32_t mask = (1 << bits) - 1, half = 1 << (bits - 1);
      o[j] = (int8_t)(((n & mask) ^ half) - half);
    }
    return;
  }
  float m = 0.0f;
  int neg = 0;
  for (uint32_t j = threadIdx.x; j < cols; j += blockDim.x) {
    float v = x[j];
    neg |= (v < 0.0f);
    m = fmaxf(m, quant == 0 ? fabsf(v) : v);
  }
  if (threadIdx.x == 0) negs = 0;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_xor_sync(0xFFFFFFFFu, m, d));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  if (neg) atomicOr(&negs, 1);
  __syncthreads();
  if (threadIdx.x < 32) {
    float r = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0.0f;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) r = fmaxf(r, __shfl_xor_sync(0xFFFFFFFFu, r, d));
    if (threadIdx.x == 0) red[0] = r;
  }
  __syncthreads();
  const float mm = red[0];  // max |x| (or max x)
  if (quant != 0 && negs) {
    if (threadIdx.x == 0) atomicOr(status + blockIdx.x, ST_QUERY);
    for (uint32_t j = threadIdx.x; j < cols; j += blockDim.x) o[j] = 0;
    return;
  }
  const int32_t M = quant == 0 ? ((1 << bits) - 1) / 2 : (1 << bits) - 1;
  const int32_t lo = quant == 0 ? -M - 1 : 0;
  for (uint32_t j = threadIdx.x; j < cols; j += blockDim.x) {
    int32_t q = 0;
    if (mm != 0.0f) {
      q = qx::round_scaled(x[j], mm, M);  // the float64 arithmetic of numpy, in integers
      q = q < lo ? lo : (q > M ? M : q);
    }
    o[j] = (int8_t)(uint8_t)(uint32_t)q;
  }
}

// ---------------------------------------------------------------------------------------------
// block helpers
// ---------------------------------------------------------------------------------------------
constexpr int kHistBins = 2048;
constexpr int kThrILP = 4;  // keys in flight per thread in the threshold passes
constexpr int kThreadsThr = 512;  // at most 64 registers: two CTAs per SM, a 256-query batch in one wave

// Largest bin b with sum(hist[b..]) >= need; *above = sum(hist[b+1..]).  Executed by warp 0.
__device__ __forceinline__ void warp_find_suffix_bin(const uint32_t* hist, int nbins,
                                                     uint32_t need, int* bin_out,
                                                     uint32_t* above_out) {
  const uint32_t lane = threadIdx.x & 31u;
  const int per = nbins / 32;
  // lane l owns bins [l*per, (l+1)*per); suffix sums from the top
  uint32_t own = 0;
  for (int i = 0; i < per; i++) own += hist[lane * per + i];
  // exclusive suffix over lanes: sum of lanes > l
  uint32_t incl = own;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t u = __shfl_down_sync(0xFFFFFFFFu, incl, d);
    if (lane + d < 32) incl += u;
  }
  uint32_t excl = incl - own;  // bins above this lane's chunk
  // the chunk holding the boundary: excl < need <= incl
  bool mine = (excl < need) && (incl >= need);
  uint32_t msk = __ballot_sync(0xFFFFFFFFu, mine);
  if (msk == 0) {  // need exceeds the total: take everything
    if (lane == 0) { *bin_out = 0; *above_out = 0; }
    return;
  }
  uint32_t owner = __ffs(msk) - 1;
  if (lane == owner) {
    uint32_t acc = excl;
    int b = (int)(lane * per + per - 1);
    for (; b >= (int)(lane * per); b--) {
      uint32_t h = hist[b];
      if (acc + h >= need) break;
      acc += h;
    }
    *bin_out = b;
    *above_out = acc;
  }
}

// ---------------------------------------------------------------------------------------------
// k_threshold: per (query, partition), a lower bound L of the r-th largest sample key (exact
// within 2^shift2), so that every row at or above the partition's Top-CK boundary has a key
// >= L with overwhelming probability; a miss is detected later (ST_MISS) and repaired.
// Also resets the partition's survivor counter.
// ---------------------------------------------------------------------------------------------
// Sample keys of query q: keys[base(q) + i * stride] with base(q) = q * ld_keys and stride 1
// (one query per pass), or, when qblk > 0 (batched passes of qblk queries),
// base(q) = (q / qblk) * qblk * ld_keys + q % qblk and stride qblk.
__global__ void __launch_bounds__(kThreadsThr, 2) k_threshold(const uint32_t* __restrict__ keys_all, uint32_t ld_keys, uint32_t qblk,
                            const uint32_t* __restrict__ part_begin, uint32_t split,
                            const uint32_t* __restrict__ r_part, uint32_t* __restrict__ thr,
                            uint32_t* __restrict__ cnt) {
  __shared__ uint32_t hist[kHistBins];
  __shared__ uint32_t smin[32], smax[32];
  __shared__ int s_bin;
  __shared__ uint32_t s_above;
  const uint32_t p = blockIdx.x, q = blockIdx.y;
  const uint32_t stride = qblk ? qblk : 1u;
  const uint32_t* kb = keys_all + (qblk ? (size_t)(q / qblk) * qblk * ld_keys + q % qblk
                                        : (size_t)q * ld_keys);
  struct Strided {
    const uint32_t* b;
    uint32_t s;
    __device__ __forceinline__ uint32_t operator[](uint32_t i) const { return b[(size_t)i * s]; }
  } kk{kb, stride};
  const uint32_t a = part_begin[p], b = part_begin[p + 1];
  const uint32_t n = b - a;
  const uint32_t r = r_part[p];
  uint32_t* T = thr + (size_t)q * split + p;
  if (threadIdx.x == 0) cnt[(size_t)q * split + p] = 0;
  if (n < r || r == 0) {
    if (threadIdx.x == 0) *T = 0;  // too few samples: keep every row of the partition
    return;
  }
  // every pass reads kThrILP keys per thread before using them: the loops are bound by global
  // load latency otherwise
  uint32_t mn = 0xFFFFFFFFu, mx = 0;
  for (uint32_t i0 = a; i0 < b; i0 += blockDim.x * kThrILP) {
    uint32_t v[kThrILP];
#pragma unroll
    for (int u = 0; u < kThrILP; u++) {
      const uint32_t i = i0 + u * blockDim.x + threadIdx.x;
      v[u] = i < b ? kk[i] : kk[a];
    }
#pragma unroll
    for (int u = 0; u < kThrILP; u++) {
      mn = min(mn, v[u]);
      mx = max(mx, v[u]);
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    mn = min(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, d));
    mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, d));
  }
  if ((threadIdx.x & 31) == 0) { smin[threadIdx.x >> 5] = mn; smax[threadIdx.x >> 5] = mx; }
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t nw = (blockDim.x + 31) / 32;
    mn = threadIdx.x < nw ? smin[threadIdx.x] : 0xFFFFFFFFu;
    mx = threadIdx.x < nw ? smax[threadIdx.x] : 0u;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      mn = min(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, d));
      mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, d));
    }
    if (threadIdx.x == 0) { smin[0] = mn; smax[0] = mx; }
  }
  __syncthreads();
  mn = smin[0];
  mx = smax[0];
  const uint32_t span = mx - mn;
  if (span == 0) {
    if (threadIdx.x == 0) *T = mn;
    return;
  }
  const int bl = 32 - __clz(span);           // bits of span
  const int sh1 = bl > 11 ? bl - 11 : 0;
  for (int i = threadIdx.x; i < kHistBins; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (uint32_t i0 = a; i0 < b; i0 += blockDim.x * kThrILP) {
    uint32_t v[kThrILP];
#pragma unroll
    for (int u = 0; u < kThrILP; u++) {
      const uint32_t i = i0 + u * blockDim.x + threadIdx.x;
      v[u] = i < b ? kk[i] : 0u;
    }
#pragma unroll
    for (int u = 0; u < kThrILP; u++) {
      const uint32_t i = i0 + u * blockDim.x + threadIdx.x;
      if (i < b) atomicAdd(&hist[(v[u] - mn) >> sh1], 1u);
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) warp_find_suffix_bin(hist, kHistBins, r, &s_bin, &s_above);
  __syncthreads();
  const uint32_t b1 = (uint32_t)s_bin, above1 = s_above;
  if (sh1 == 0) {
    if (threadIdx.x == 0) *T = mn + b1;
    return;
  }
  const int sh2 = sh1 > 11 ? sh1 - 11 : 0;
  __syncthreads();
  for (int i = threadIdx.x; i < kHistBins; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (uint32_t i0 = a; i0 < b; i0 += blockDim.x * kThrILP) {
    uint32_t v[kThrILP];
#pragma unroll
    for (int u = 0; u < kThrILP; u++) {
      const uint32_t i = i0 + u * blockDim.x + threadIdx.x;
      v[u] = i < b ? kk[i] : 0u;
    }
#pragma unroll
    for (int u = 0; u < kThrILP; u++) {
      const uint32_t i = i0 + u * blockDim.x + threadIdx.x;
      if ((i < b) && (((v[u] - mn) >> sh1) == b1))
        atomicAdd(&hist[((v[u] - mn) >> sh2) & ((1u << (sh1 - sh2)) - 1u)], 1u);
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) warp_find_suffix_bin(hist, kHistBins, r - above1, &s_bin, &s_above);
  __syncthreads();
  if (threadIdx.x == 0) *T = mn + (b1 << sh1) + ((uint32_t)s_bin << sh2);
}

// ---------------------------------------------------------------------------------------------
// Block-wide exact select: the `need` largest 64-bit composites (key << 32 | row) of n items.
// Items come from an accessor; returns through smem the threshold composite tau such that
// exactly `need` items are >= tau (composites are unique because rows are).
// ---------------------------------------------------------------------------------------------
template <class Get>
__device__ uint64_t block_select_tau(Get get, uint32_t n, uint32_t need, uint32_t* hist256,
                                     uint64_t* sh64) {
  // min / max composite
  uint64_t mn = ~0ull, mx = 0;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    uint64_t c = get(i);
    mn = c < mn ? c : mn;
    mx = c > mx ? c : mx;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    uint64_t a = __shfl_xor_sync(0xFFFFFFFFu, mn, d), b = __shfl_xor_sync(0xFFFFFFFFu, mx, d);
    mn = a < mn ? a : mn;
    mx = b > mx ? b : mx;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { sh64[threadIdx.x >> 5] = mn; sh64[32 + (threadIdx.x >> 5)] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t nw = (blockDim.x + 31) / 32;
    uint64_t a = ~0ull, b = 0;
    for (uint32_t w = 0; w < nw; w++) {
      a = sh64[w] < a ? sh64[w] : a;
      b = sh64[32 + w] > b ? sh64[32 + w] : b;
    }
    sh64[64] = a;
    sh64[65] = b;
  }
  __syncthreads();
  mn = sh64[64];
  mx = sh64[65];
  if (need >= n) return mn;
  if (mn == mx) return mn;
  int hi = 63 - __clzll((long long)(mn ^ mx));
  uint64_t prefix = mx & ~((hi == 63) ? ~0ull : ((2ull << hi) - 1ull));
  uint64_t fixed = ~((hi == 63) ? ~0ull : ((2ull << hi) - 1ull));
  uint32_t need_rem = need;
  while (true) {
    const int lo = hi >= 7 ? hi - 7 : 0;
    const int width = hi - lo + 1;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist256[i] = 0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      uint64_t c = get(i);
      if ((c & fixed) == prefix)
        atomicAdd(&hist256[(uint32_t)(c >> lo) & ((1u << width) - 1u)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      // 256 bins, 8 per lane
      const uint32_t lane = threadIdx.x;
      uint32_t own = 0;
      for (int i = 0; i < 8; i++) own += hist256[lane * 8 + i];
      uint32_t incl = own;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t u = __shfl_down_sync(0xFFFFFFFFu, incl, d);
        if (lane + d < 32) incl += u;
      }
      uint32_t excl = incl - own;
      bool mine = (excl < need_rem) && (incl >= need_rem);
      uint32_t msk = __ballot_sync(0xFFFFFFFFu, mine);
      uint32_t owner = msk ? (__ffs(msk) - 1) : 0;
      if (lane == owner) {
        uint32_t acc = excl;
        int bb = lane * 8 + 7;
        for (; bb > (int)(lane * 8); bb--) {
          if (acc + hist256[bb] >= need_rem) break;
          acc += hist256[bb];
        }
        sh64[66] = (uint64_t)bb;
        sh64[67] = (uint64_t)acc;
        sh64[68] = (uint64_t)hist256[bb];
      }
    }
    __syncthreads();
    const uint32_t d = (uint32_t)sh64[66];
    const uint32_t above = (uint32_t)sh64[67];
    const uint32_t inbin = (uint32_t)sh64[68];
    __syncthreads();
    need_rem -= above;
    prefix |= (uint64_t)d << lo;
    fixed |= (uint64_t)((1u << width) - 1u) << lo;
    if (inbin == need_rem || lo == 0) break;
    hi = lo - 1;
  }
  return prefix;
}

// ---------------------------------------------------------------------------------------------
// k_select: per (query, partition) exact Top-ntop of the survivors by (key desc, row desc).
// implicit = true reads every row of the partition from a full key array (slow path).
// ---------------------------------------------------------------------------------------------
struct SelectArgs {
  const uint2* surv;        // [nq][split][cap]
  const uint32_t* cnt;      // [nq][split]
  uint32_t cap;
  const uint32_t* allkeys;  // implicit: [n_rows] keys of query `q0`
  uint32_t q0;
  uint32_t split, slice, n_rows, ntop;
  uint32_t* cand;           // [nq][split*ntop] rows, 0xFFFFFFFF = empty slot
  uint32_t* cand_key;       // [nq][split*ntop]
  uint32_t* status;         // [nq]
};

template <bool IMPLICIT>
__global__ void k_select(SelectArgs a) {
  __shared__ uint32_t hist[256];
  __shared__ uint64_t sh64[72];
  __shared__ uint32_t s_out;
  const uint32_t p = blockIdx.x, q = IMPLICIT ? a.q0 : blockIdx.y;
  const uint32_t r0 = p * a.slice;
  const uint32_t r1 = (a.split <= 1 || p == a.split - 1) ? a.n_rows : (p + 1) * a.slice;
  const uint32_t prow = (a.split <= 1) ? a.n_rows : (r1 - r0);
  const uint32_t need = min(a.ntop, prow);
  uint32_t* cr = a.cand + ((size_t)q * a.split + p) * a.ntop;
  uint32_t* ck = a.cand_key + ((size_t)q * a.split + p) * a.ntop;
  for (uint32_t i = threadIdx.x; i < a.ntop; i += blockDim.x) { cr[i] = 0xFFFFFFFFu; ck[i] = 0; }
  uint32_t n;
  if (IMPLICIT) {
    n = (a.split <= 1) ? a.n_rows : prow;
  } else {
    n = a.cnt[(size_t)q * a.split + p];
    if (n > a.cap) {
      if (threadIdx.x == 0) atomicOr(a.status + q, ST_OVERFLOW);
      return;
    }
    if (n < need) {
      if (threadIdx.x == 0) atomicOr(a.status + q, ST_MISS);
      return;
    }
  }
  const uint32_t base = (a.split <= 1) ? 0 : r0;
  const uint2* sv = a.surv + ((size_t)q * a.split + p) * a.cap;
  auto get = [&](uint32_t i) -> uint64_t {
    if (IMPLICIT) {
      uint32_t row = base + i;
      return ((uint64_t)a.allkeys[row] << 32) | row;
    } else {
      uint2 v = sv[i];
      return ((uint64_t)v.x << 32) | v.y;
    }
  };
  __syncthreads();
  if (need == 0) return;
  const uint64_t tau = block_select_tau(get, n, need, hist, sh64);
  if (threadIdx.x == 0) s_out = 0;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    uint64_t c = get(i);
    if (c >= tau) {
      uint32_t o = atomicAdd(&s_out, 1u);
      if (o < a.ntop) {
        cr[o] = (uint32_t)c;
        ck[o] = (uint32_t)(c >> 32);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// k_final: FP32 rescoring of every candidate (sequential over the row's entries in column
// order, separately rounded multiply and add) and the final Top-K in sort_tuples order.
// One CTA per query. Each warp rescores 32 slots at a time: it loads its rows' entries row by
// row (lane = entry, coalesced, 8 rows in flight), stages the rounded products in shared memory
// and each lane then sums its own row's products in entry order. The K largest (score, row)
// composites are found by a block radix select, then only those are sorted by a bitonic network
// in shared memory.
// ---------------------------------------------------------------------------------------------
struct FinalArgs {
  const uint32_t* csr_ptr;   // [rows+1]
  const uint16_t* csr_col;
  const float* csr_val;
  const float* q32;          // [nq][ld32]
  uint32_t ld32, cols;
  const uint32_t* cand;      // [nq][nslots]
  uint32_t nslots, kp, k;    // kp: power of two >= k
  uint32_t* out_idx;         // [nq][k]
  float* out_score;          // [nq][k]
  const uint32_t* status;    // [nq]; queries with a set status are left to the repair path
  // [nq][nslots] candidate keys, or null.  Given: the final Top-K ranks the candidates by their
  // integer candidate score (no FP32 rescoring: a pre-quantised matrix or query without FP32
  // values) and out_score holds that score
  const uint32_t* cand_key;
};

constexpr int kThreadsFinal = 512;  // two CTAs per SM: a 256-query batch runs in one wave
constexpr int kFinalStageLd = 33;   // staged products: 32 rows x 33 floats per warp

// dynamic shared memory of k_final: the query, the composites of all slots, then one region
// holding first the per-warp product staging and afterwards the kp selected composites
__host__ __device__ inline size_t final_smem_bytes(uint32_t cols, uint32_t nslots, uint32_t kp) {
  const size_t stage = (size_t)(kThreadsFinal / 32) * 32 * kFinalStageLd * 4;
  const size_t top = (size_t)kp * 8;
  return (((size_t)cols * 4 + 15) & ~(size_t)15) + (size_t)nslots * 8 + (stage > top ? stage : top);
}

__global__ void __launch_bounds__(kThreadsFinal, 2) k_final(FinalArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t hist[256];
  __shared__ uint64_t sh64[72];
  __shared__ uint32_t s_cnt;
  float* qs = reinterpret_cast<float*>(smem);
  uint64_t* comp = reinterpret_cast<uint64_t*>(smem + ((a.cols * 4 + 15) & ~15u));
  uint64_t* top = comp + a.nslots;  // after the rescoring; the product staging before it
  const uint32_t q = blockIdx.x;
  if (a.status && a.status[q]) return;
  if (!a.cand_key) {
    const float* x = a.q32 + (size_t)q * a.ld32;
    for (uint32_t j = threadIdx.x; j < a.cols; j += blockDim.x) qs[j] = x[j];
  }
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  const uint32_t* cr = a.cand + (size_t)q * a.nslots;
  if (a.cand_key) {  // integer ranking: the candidate keys themselves
    const uint32_t* ck = a.cand_key + (size_t)q * a.nslots;
    for (uint32_t i = threadIdx.x; i < a.nslots; i += blockDim.x) {
      const uint32_t row = cr[i];
      comp[i] = row != 0xFFFFFFFFu ? ((uint64_t)ck[i] << 32) | row : 0ull;
    }
  } else {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    float* sp = reinterpret_cast<float*>(top) + warp * (32 * kFinalStageLd);
    for (uint32_t g = warp * 32; g < a.nslots; g += nwarps * 32) {
      const uint32_t i = g + lane;
      const uint32_t row = i < a.nslots ? cr[i] : 0xFFFFFFFFu;
      uint32_t s = 0, n = 0;
      if (row != 0xFFFFFFFFu) {
        s = a.csr_ptr[row];
        n = a.csr_ptr[row + 1] - s;
      }
      const uint32_t rounds = (__reduce_max_sync(0xFFFFFFFFu, n) + 31) >> 5;
      float acc = 0.0f;
      for (uint32_t r = 0; r < rounds; r++) {
        const uint32_t o = r * 32 + lane;
#pragma unroll 8
        for (int j = 0; j < 32; j++) {
          const uint32_t sj = __shfl_sync(0xFFFFFFFFu, s, j), nj = __shfl_sync(0xFFFFFFFFu, n, j);
          float p = 0.0f;
          if (o < nj) p = __fmul_rn(__ldg(a.csr_val + sj + o), qs[__ldg(a.csr_col + sj + o)]);
          sp[j * kFinalStageLd + lane] = p;
        }
        __syncwarp();
        const uint32_t m = n > r * 32 ? min(n - r * 32, 32u) : 0u;
        for (uint32_t e = 0; e < m; e++) acc = __fadd_rn(acc, sp[lane * kFinalStageLd + e]);
        __syncwarp();
      }
      if (i < a.nslots) comp[i] = row != 0xFFFFFFFFu ? ((uint64_t)key_f32(acc) << 32) | row : 0ull;
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < a.kp; i += blockDim.x) top[i] = 0;
  // composites of filled slots are unique (rows are); empty slots are 0 and never selected
  const uint32_t need = min(a.k, a.nslots);
  const uint64_t tau = block_select_tau([&](uint32_t i) -> uint64_t { return comp[i]; }, a.nslots,
                                        need, hist, sh64);
  for (uint32_t i = threadIdx.x; i < a.nslots; i += blockDim.x) {
    const uint64_t c = comp[i];
    if (c != 0 && c >= tau) {
      const uint32_t o = atomicAdd(&s_cnt, 1u);
      if (o < a.kp) top[o] = c;
    }
  }
  __syncthreads();
  // bitonic sort of the kp selected composites, descending
  for (uint32_t kk = 2; kk <= a.kp; kk <<= 1) {
    for (uint32_t j = kk >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < a.kp; i += blockDim.x) {
        uint32_t l = i ^ j;
        if (l > i) {
          uint64_t ci = top[i], cl = top[l];
          bool desc = ((i & kk) == 0);
          if (desc ? (ci < cl) : (ci > cl)) { top[i] = cl; top[l] = ci; }
        }
      }
      __syncthreads();
    }
  }
  for (uint32_t i = threadIdx.x; i < a.k; i += blockDim.x) {
    uint64_t c = (i < a.kp) ? top[i] : 0;
    uint32_t* oi = a.out_idx + (size_t)q * a.k;
    float* os = a.out_score + (size_t)q * a.k;
    if (c == 0) {
      oi[i] = 0xFFFFFFFFu;
      os[i] = -__int_as_float(0x7f800000);
    } else {
      oi[i] = (uint32_t)c;
      const uint32_t key = (uint32_t)(c >> 32);
      os[i] = a.cand_key ? (float)(int32_t)(key ^ 0x80000000u) : key_to_f32(key);
    }
  }
}

}  // namespace dev
}  // namespace aes

namespace aes {
namespace dev {

// FP32-only pass: the FP32 score of every row (each row summed in column order with separately
// rounded multiply and add: spmv_coo_gold_top_k, gold_algorithms.hpp:189-247 with V = float) as an
// order-preserving key.  A warp takes 32 consecutive rows, one per lane.  Their entries are
// contiguous in the CSR, so the warp walks them in chunks of kExactChunk: every lane loads entries
// of the chunk (coalesced, all loads in flight at once) and stores their rounded products
// v * q[col] to shared memory in entry order; then each lane adds its own row's products of the
// chunk in order.  The products and the order of the additions are those of the sequential sum.
constexpr uint32_t kExactChunk = 512;       // entries per warp and chunk
constexpr uint32_t kExactWarps = 8;         // warps per CTA
__host__ inline size_t exact_all_smem_bytes(uint32_t cols) {
  return (size_t)cols * 4 + (size_t)kExactWarps * kExactChunk * 4;
}

__global__ void __launch_bounds__(kExactWarps * 32) k_exact_all(
    const uint32_t* __restrict__ ptr, const uint16_t* __restrict__ col,
    const float* __restrict__ val, const float* __restrict__ q, uint32_t cols, uint32_t rows,
    uint32_t* __restrict__ keys) {
  extern __shared__ __align__(16) unsigned char xsm[];
  float* qs = reinterpret_cast<float*>(xsm);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  float* sp = reinterpret_cast<float*>(xsm + (size_t)cols * 4) + warp * kExactChunk;
  for (uint32_t j = threadIdx.x; j < cols; j += blockDim.x) qs[j] = q[j];
  __syncthreads();
  const uint32_t nblk = (rows + 31) / 32;
  for (uint32_t blk = blockIdx.x * kExactWarps + warp; blk < nblk; blk += gridDim.x * kExactWarps) {
    const uint32_t r0 = blk * 32, r = r0 + lane;
    const uint32_t rend = min(r0 + 32u, rows);
    const uint32_t E0 = ptr[r0], E1 = ptr[rend];
    const uint32_t s = r < rows ? ptr[r] : E1, e = r < rows ? ptr[r + 1] : E1;
    float acc = 0.0f;
    for (uint32_t c = E0; c < E1; c += kExactChunk) {
      const uint32_t n = min(kExactChunk, E1 - c);
      float lv[kExactChunk / 32];
      uint32_t lc[kExactChunk / 32];
#pragma unroll
      for (uint32_t u = 0; u < kExactChunk / 32; u++) {
        const uint32_t i = u * 32 + lane;
        lv[u] = i < n ? __ldcs(val + c + i) : 0.0f;
        lc[u] = i < n ? (uint32_t)__ldcs(col + c + i) : 0u;
      }
#pragma unroll
      for (uint32_t u = 0; u < kExactChunk / 32; u++) sp[u * 32 + lane] = __fmul_rn(lv[u], qs[lc[u]]);
      __syncwarp();
      const uint32_t a = max(s, c), b = min(e, c + n);
      for (uint32_t i = a; i < b; i++) acc = __fadd_rn(acc, sp[i - c]);
      __syncwarp();
    }
    if (r < rows) keys[r] = key_f32(acc);
  }
}

// Rows whose key is at least *thr, appended as (key, row) to surv (warp-aggregated counter; the
// count goes on past cap so the select can tell an overflow).  Used by the FP32-only pass after
// a sample threshold, so that the select reads a few survivors instead of every row.
__global__ void k_filter_keys(const uint32_t* __restrict__ keys, uint32_t rows,
                              const uint32_t* __restrict__ thr, uint32_t* __restrict__ cnt,
                              uint2* __restrict__ surv, uint32_t cap) {
  const uint32_t th = *thr, lane = threadIdx.x & 31u;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t n4 = (rows + 3) / 4;                    // groups of four keys (16-byte loads)
  const uint32_t n_iter = (n4 + stride - 1) / stride;    // the same for every lane of a warp
  for (uint32_t it = 0; it < n_iter; it++) {
    const uint32_t g = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t k4[4] = {0u, 0u, 0u, 0u};
    if (g * 4 + 3 < rows) {
      const uint4 v = __ldcs(reinterpret_cast<const uint4*>(keys) + g);
      k4[0] = v.x; k4[1] = v.y; k4[2] = v.z; k4[3] = v.w;
    } else if (g < n4) {
      for (uint32_t t = 0; t < 4 && g * 4 + t < rows; t++) k4[t] = keys[g * 4 + t];
    }
#pragma unroll
    for (uint32_t t = 0; t < 4; t++) {
      const uint32_t r = g * 4 + t;
      const bool hit = r < rows && k4[t] >= th;
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, hit);
      if (m) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(cnt, (uint32_t)__popc(m));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (hit) {
          const uint32_t i = base + __popc(m & ((1u << lane) - 1u));
          if (i < cap) surv[i] = make_uint2(k4[t], r);
        }
      }
    }
  }
}

}  // namespace dev
}  // namespace aes
