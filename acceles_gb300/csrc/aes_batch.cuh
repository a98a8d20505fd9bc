// aes_batch.cuh -- batched candidate pass: one read of the Ultra-CSR matrix scores a block of up
// to 128 queries (the reference's spmv_ucsr_top_k_main scores one query per pass,
// spmv_ucsr_top_k_multicore.cpp:8-143).  One launch scores every block of a batch: blockIdx.y
// is the block, so the blocks run as successive waves of CTAs, each CTA loading its block's
// query table once.
//
// Per warp and 32-packet tile:
//   phase A (lane = packet): decode the packet's flags, 10-bit columns and B-bit values into
//            per-warp shared records in element order;
//   phase B (lane = 4 queries): walk the tile's elements four at a time.  For a group of four
//            elements every lane gathers its four queries' bytes at the four columns (one 32-bit
//            load each from the query table, 33 words per column: lane l's word at col * 33 + l,
//            so a gather is conflict-free and its address one multiply-add), transposes the 4x4
//            bytes with PRMT and accumulates with dp4a (exact int8 x int8 -> int32).  Row flags
//            are the same for every lane, so row boundaries never diverge.
#pragma once

#include "aes_kernels.cuh"

namespace aes {
namespace dev {

constexpr int kBatchQ = 128;         // queries per tile (32 lanes x 4)
constexpr uint32_t kQtabWords = 33;  // query table words per column: 32 lanes and a pad word
// words of one block's query table, padded to whole 16-byte slots
__host__ __device__ constexpr size_t batch_qtab_words(uint32_t cols) {
  return ((size_t)cols * kQtabWords + 3) & ~(size_t)3;
}
constexpr int kWarpsBatchMax = 16;
constexpr size_t kSmemMax = 227 * 1024;

struct BatchArgs {
  const uint4* tiles;
  const uint32_t* tile_rowbase;
  uint32_t n_tiles, n_rows, cols;
  const uint32_t* qtab;         // [blocks][cols][33] words: bytes of queries 128 b + 4l .. 4l+3 at
                                // (col, lane l)
  uint32_t nq;                  // queries of the batch (blocks = ceil(nq / 128))
  uint32_t blk0;                // blocks blk0 .. blk0 + gridDim.y - 1 in this launch
  const float* rowscale;
  uint32_t split, slice;
  const uint32_t* thr;          // [nq][split] (MODE_FILTER)
  uint32_t* cnt;                // [nq][split]
  uint2* surv;                  // [nq][split][cap]
  uint32_t cap;
  uint32_t* keys_out;           // MODE_SAMPLE: block b at keys_out + b * 128 * n_sample_rows,
                                // [sample rows][128]
  const uint32_t* sample_first;
  uint32_t sample_stride, n_sample_tiles, n_sample_rows;
};

// per-warp element records: columns (u32), values (u8) and row flags (u8) of the 32
// packets of a tile, plus one zero group of four so the walk can read one group ahead
template <int B>
__host__ __device__ constexpr uint32_t batch_rec_elems() {
  return 32u * packet_elems(B) + 4u;
}
template <int B>
__host__ __device__ constexpr size_t batch_warp_bytes() {
  return ((size_t)batch_rec_elems<B>() * 6 + 15) & ~(size_t)15;
}
__host__ __device__ constexpr size_t batch_warp_bytes_rt(int B) {
  return (((size_t)32 * packet_elems(B) + 4) * 6 + 15) & ~(size_t)15;
}

__host__ __device__ inline bool batch_thr_in_smem(uint32_t split) { return split > 1 && split <= 32; }

// warps per CTA that fit next to the query table (and thresholds) in shared memory
__host__ inline int batch_warps(int B, uint32_t cols, uint32_t split) {
  const size_t per = batch_warp_bytes_rt(B);
  const size_t fixed = batch_qtab_words(cols) * 4 + (batch_thr_in_smem(split) ? (size_t)split * kBatchQ * 4 : 0);
  int w = (int)((kSmemMax - fixed) / per);
  return w > kWarpsBatchMax ? kWarpsBatchMax : w;
}
__host__ inline size_t batch_smem_bytes(int B, uint32_t cols, uint32_t split, int warps) {
  const size_t per = batch_warp_bytes_rt(B);
  return batch_qtab_words(cols) * 4 + (batch_thr_in_smem(split) ? (size_t)split * kBatchQ * 4 : 0) +
         (size_t)warps * per;
}

// 4x4 byte transpose: V[t] byte i = W[i] byte t
__device__ __forceinline__ void transpose4(const uint32_t (&W)[4], uint32_t (&V)[4]) {
  const uint32_t x0 = __byte_perm(W[0], W[1], 0x5140);
  const uint32_t x1 = __byte_perm(W[0], W[1], 0x7362);
  const uint32_t y0 = __byte_perm(W[2], W[3], 0x5140);
  const uint32_t y1 = __byte_perm(W[2], W[3], 0x7362);
  V[0] = __byte_perm(x0, y0, 0x5410);
  V[1] = __byte_perm(x0, y0, 0x7632);
  V[2] = __byte_perm(x1, y1, 0x5410);
  V[3] = __byte_perm(x1, y1, 0x7632);
}

template <bool SGN>
__device__ __forceinline__ int32_t dot4(uint32_t a, uint32_t b, int32_t c) {
  if constexpr (SGN) return __dp4a((int)a, (int)b, c);
  else return (int32_t)__dp4a(a, b, (unsigned)c);
}

template <int MODE>
struct BatchRows {
  const BatchArgs& a;
  const uint32_t* thr_s;  // [split][128] in smem (split in 2..64), else nullptr
  uint32_t thr4[4];       // split == 1
  int32_t thr_sc[4];      // split == 1, integer keys: thr4 as signed score bounds
  uint32_t sample_base;
  uint32_t lane;
  uint32_t q0, nq;        // the block's queries q0 .. q0 + nq - 1
  uint32_t* keys_blk;     // MODE_SAMPLE: the block's key array

  // the four queries of this lane finished row `row` with integer scores acc[0..3]
  __device__ __forceinline__ void finish(uint32_t row, const int32_t (&acc)[4]) const {
    if constexpr (MODE == MODE_FILTER) {
      if (!a.rowscale && a.split <= 1) {
        // integer keys, one partition: key >= th  <=>  score >= th ^ 0x80000000 (signed)
        const bool hit = (acc[0] >= thr_sc[0]) | (acc[1] >= thr_sc[1]) | (acc[2] >= thr_sc[2]) |
                         (acc[3] >= thr_sc[3]);
        if (__ballot_sync(0xFFFFFFFFu, hit)) append(row, 0, acc, thr4, false);
        return;
      }
    }
    uint32_t key[4];
    if (a.rowscale) {
      const float rs = __ldg(a.rowscale + row);
#pragma unroll
      for (int t = 0; t < 4; t++) key[t] = key_f32(__fmul_rn(__int2float_rn(acc[t]), rs));
    } else {
#pragma unroll
      for (int t = 0; t < 4; t++) key[t] = key_i32(acc[t]);
    }
    if constexpr (MODE == MODE_SAMPLE) {
      reinterpret_cast<uint4*>(keys_blk)[(size_t)(row - sample_base) * 32 + lane] =
          make_uint4(key[0], key[1], key[2], key[3]);
    } else if constexpr (MODE == MODE_FILTER) {
      const uint32_t p = part_of(row, a.split, a.slice);
      uint32_t th[4];
      if (a.split <= 1) {
#pragma unroll
        for (int t = 0; t < 4; t++) th[t] = thr4[t];
      } else if (thr_s) {
        const uint4 v = reinterpret_cast<const uint4*>(thr_s)[p * 32 + lane];
        th[0] = v.x; th[1] = v.y; th[2] = v.z; th[3] = v.w;
      } else {
#pragma unroll
        for (int t = 0; t < 4; t++) {
          const uint32_t q = 4 * lane + t;
          th[t] = q < nq ? __ldg(a.thr + (size_t)(q0 + q) * a.split + p) : 0xFFFFFFFFu;
        }
      }
      const bool hit = (key[0] >= th[0]) | (key[1] >= th[1]) | (key[2] >= th[2]) | (key[3] >= th[3]);
      if (__ballot_sync(0xFFFFFFFFu, hit)) {
        int32_t k2[4];
#pragma unroll
        for (int t = 0; t < 4; t++) k2[t] = (int32_t)key[t];
        append(row, p, k2, th, true);
      }
    }
  }

  // key threshold of partition p for this lane's query t
  __device__ __forceinline__ uint32_t thr_q(uint32_t p, int t) const {
    if (a.split <= 1) return thr4[t];
    if (thr_s) return thr_s[p * kBatchQ + 4 * lane + t];
    const uint32_t q = 4 * lane + t;
    return q < nq ? __ldg(a.thr + (size_t)(q0 + q) * a.split + p) : 0xFFFFFFFFu;
  }
  // integer keys: per query, the lowest score bound over the partitions of rows r0 .. r1 (one
  // partition for almost every tile: the partitions are contiguous row ranges)
  __device__ __forceinline__ void bounds(uint32_t r0, uint32_t r1, int32_t (&b)[4]) const {
    if (a.split <= 1) {
#pragma unroll
      for (int t = 0; t < 4; t++) b[t] = thr_sc[t];
      return;
    }
#pragma unroll
    for (int t = 0; t < 4; t++) b[t] = 0x7FFFFFFF;
    const uint32_t p1 = part_of(r1, a.split, a.slice);
    for (uint32_t p = part_of(r0, a.split, a.slice); p <= p1; p++) {
#pragma unroll
      for (int t = 0; t < 4; t++) b[t] = min(b[t], (int32_t)(thr_q(p, t) ^ 0x80000000u));
    }
  }
  // integer keys: row `row` finished with scores acc[0..3]; bound b from bounds()
  __device__ __forceinline__ void finish_int(uint32_t row, const int32_t (&acc)[4],
                                             const int32_t (&b)[4]) const {
    const bool hit = (acc[0] >= b[0]) | (acc[1] >= b[1]) | (acc[2] >= b[2]) | (acc[3] >= b[3]);
    if (__ballot_sync(0xFFFFFFFFu, hit)) {
      const uint32_t p = part_of(row, a.split, a.slice);
      uint32_t th[4];
#pragma unroll
      for (int t = 0; t < 4; t++) th[t] = thr_q(p, t);
      append(row, p, acc, th, false);
    }
  }

  // survivors of a finished row (rare): v[t] is the key (is_key) or the integer score
  __device__ __forceinline__ void append(uint32_t row, uint32_t p, const int32_t (&v)[4],
                                      const uint32_t (&th)[4], bool is_key) const {
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const uint32_t key = is_key ? (uint32_t)v[t] : key_i32(v[t]);
      const uint32_t q = 4 * lane + t;
      if (key >= th[t] && q < nq) {
        const size_t qp = (size_t)(q0 + q) * a.split + p;
        const uint32_t i = atomicAdd(a.cnt + qp, 1u);
        if (i < a.cap) a.surv[qp * a.cap + i] = make_uint2(key, row);
      }
    }
  }
};

template <int B, bool SGN, int MODE>
__device__ void batch_range(const BatchArgs& a, uint32_t tb, uint32_t te,
                            const BatchRows<MODE>& rows, const uint8_t* qtb,
                            unsigned char* wsm) {
  constexpr int P = packet_elems(B);
  constexpr int NE = 32 * P;                 // elements per tile
  constexpr int NG = NE / 4;                 // groups of four
  constexpr uint32_t NR = batch_rec_elems<B>();
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lane4 = lane << 2;
  constexpr uint32_t RB = kQtabWords * 4;  // query table bytes per column
  uint32_t* offs = reinterpret_cast<uint32_t*>(wsm);            // [NR] col
  uint8_t* vals = wsm + (size_t)NR * 4;                          // [NR]
  uint8_t* flg = wsm + (size_t)NR * 5;                           // [NR]
  if (tb >= te) return;
  bool owned = (tb == 0);
  uint32_t row = __ldg(a.tile_rowbase + tb);  // id of the row open before the first entry
  int32_t acc[4] = {0, 0, 0, 0};
  uint32_t w[16], nw[16];
  load_tile(a.tiles, tb, lane, w);
  for (uint32_t t = tb;; t++) {
    if (t >= a.n_tiles) {
      if (owned) rows.finish(row, acc);
      return;
    }
    const bool closing = (t >= te);
    bool simple = owned && !closing;  // boundaries need neither the ownership nor the end test
    // integer keys: compare against the tile's per-query score bounds, exact check on a hit
    constexpr bool kIntKeysPossible = MODE == MODE_FILTER;
    const bool intk = kIntKeysPossible && !a.rowscale;
    int32_t bnd[4] = {0, 0, 0, 0};
    if (intk) {
      const uint32_t nfl = __reduce_add_sync(0xFFFFFFFFu, (uint32_t)popc_flags(PacketDecoder<B, SGN>::flags(w)));
      rows.bounds(row, row + nfl, bnd);
    }
    auto fin = [&](uint32_t r, const int32_t (&x)[4]) {
      if (kIntKeysPossible && intk) rows.finish_int(r, x, bnd);
      else rows.finish(r, x);
    };
    // prefetch one tile ahead up to the first closing tile; later tiles are read on demand
    if (t + 1 <= te && t + 1 < a.n_tiles) load_tile(a.tiles, t + 1, lane, nw);
    // ---- phase A: this lane's packet -> records ----------------------------------------------
    {
      using D = PacketDecoder<B, SGN>;
      const auto F = D::flags(w);
      uint32_t* o = offs + lane * P;
      uint8_t* v = vals + lane * P;
      uint8_t* f = flg + lane * P;
#pragma unroll
      for (int j = 0; j < P; j++) {
        const uint32_t cpos = P + 10 * j, vpos = 11 * P + B * j;
        const uint32_t cw = __funnelshift_r(w[cpos >> 5], w[(cpos >> 5) + 1 < 16 ? (cpos >> 5) + 1 : 15], cpos & 31);
        o[j] = cw & 0x3FFu;
        const uint32_t vw = __funnelshift_r(w[vpos >> 5], w[(vpos >> 5) + 1 < 16 ? (vpos >> 5) + 1 : 15], vpos & 31);
        uint32_t vb = vw & ((1u << B) - 1u);
        if (SGN) vb = (uint32_t)(((int32_t)(vb << (32 - B))) >> (32 - B)) & 0xFFu;
        v[j] = (uint8_t)vb;
        f[j] = (uint8_t)((F >> j) & 1u);
      }
    }
    __syncwarp();
    // ---- phase B: lanes = queries ------------------------------------------------------------
    // The gathers of group g+1 are issued before group g's arithmetic and branches (the zero
    // group after the last one keeps the read in bounds).  The flag word comes through a
    // shuffle from lane 0 (every lane holds the same word): branches on it are then known to be
    // warp-uniform and need no reconvergence bookkeeping.
    const uint4* O = reinterpret_cast<const uint4*>(offs);
    const uint32_t* Vg = reinterpret_cast<const uint32_t*>(vals);
    const uint32_t* Fg = reinterpret_cast<const uint32_t*>(flg);
    uint32_t Wn[4], v4n, f4n;
    {
      const uint4 o4 = O[0];
      v4n = Vg[0];
      f4n = __shfl_sync(0xFFFFFFFFu, Fg[0], 0);
      Wn[0] = *reinterpret_cast<const uint32_t*>(qtb + (o4.x * RB + lane4));
      Wn[1] = *reinterpret_cast<const uint32_t*>(qtb + (o4.y * RB + lane4));
      Wn[2] = *reinterpret_cast<const uint32_t*>(qtb + (o4.z * RB + lane4));
      Wn[3] = *reinterpret_cast<const uint32_t*>(qtb + (o4.w * RB + lane4));
    }
#pragma unroll 2
    for (int g = 0; g < NG; g++) {
      const uint32_t W[4] = {Wn[0], Wn[1], Wn[2], Wn[3]};
      const uint32_t v4 = v4n, f4 = f4n;
      {
        const uint4 o4 = O[g + 1];
        v4n = Vg[g + 1];
        f4n = __shfl_sync(0xFFFFFFFFu, Fg[g + 1], 0);
        Wn[0] = *reinterpret_cast<const uint32_t*>(qtb + (o4.x * RB + lane4));
        Wn[1] = *reinterpret_cast<const uint32_t*>(qtb + (o4.y * RB + lane4));
        Wn[2] = *reinterpret_cast<const uint32_t*>(qtb + (o4.z * RB + lane4));
        Wn[3] = *reinterpret_cast<const uint32_t*>(qtb + (o4.w * RB + lane4));
      }
      uint32_t V[4];
      transpose4(W, V);
      if (f4 == 0) {
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] = dot4<SGN>(v4, V[q], acc[q]);
        continue;
      }
      if ((f4 & (f4 - 1u)) == 0) {
        // one row starts in this group, at byte i: bytes [0, i) end the open row
        const uint32_t m = (f4 & (0u - f4)) - 1u;
        const uint32_t lo = v4 & m, hi = v4 & ~m;
        int32_t s[4];
#pragma unroll
        for (int q = 0; q < 4; q++) s[q] = dot4<SGN>(lo, V[q], acc[q]);
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] = dot4<SGN>(hi, V[q], 0);
        if (simple) {  // an owned row inside the range
          fin(row, s);
          row++;
          continue;
        }
        if (owned) fin(row, s);
        if (closing) return;
        row++;
        owned = true;
        simple = true;
        continue;
      }
      // two or more rows start in this group: bit i of fm <=> element i starts a row
      uint32_t fm = (f4 * 0x01020408u) >> 24;
      uint32_t lo_mask = 0xFFFFFFFFu;  // bytes of the group not yet accumulated
      do {
        const int i = __ffs(fm) - 1;
        fm &= fm - 1;
        const uint32_t m = lo_mask & ~(0xFFFFFFFFu << (8 * i));  // bytes [lo, i)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] = dot4<SGN>(v4 & m, V[q], acc[q]);
        if (owned) fin(row, acc);
        if (closing) return;
        row++;
        owned = true;
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] = 0;
        lo_mask = 0xFFFFFFFFu << (8 * i);
      } while (fm);
      simple = true;  // owned now, and not closing (that returned above)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[q] = dot4<SGN>(v4 & lo_mask, V[q], acc[q]);
    }
    __syncwarp();
    if (t + 1 > te) {
      if (t + 1 < a.n_tiles) load_tile(a.tiles, t + 1, lane, w);
    } else {
#pragma unroll
      for (int i = 0; i < 16; i++) w[i] = nw[i];
    }
  }
}

template <int B, bool SGN, int MODE>
__global__ void __launch_bounds__(kWarpsBatchMax * 32, 1) k_cand_batch(BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint8_t* qtb = smem;                                           // [cols][33] words
  const size_t qtab_bytes = batch_qtab_words(a.cols) * 4;
  uint32_t* thr_s = reinterpret_cast<uint32_t*>(smem + qtab_bytes);
  const bool thr_in_smem = (MODE == MODE_FILTER) && batch_thr_in_smem(a.split);
  unsigned char* wsm_all = smem + qtab_bytes +
                           (batch_thr_in_smem(a.split) ? (size_t)a.split * kBatchQ * 4 : 0);
  // the warp index through a shuffle from lane 0: the compiler then treats the range bounds, and
  // every branch on them, as warp-uniform
  const uint32_t warp = __shfl_sync(0xFFFFFFFFu, threadIdx.x >> 5, 0), lane = threadIdx.x & 31u;
  unsigned char* wsm = wsm_all + (size_t)warp * batch_warp_bytes<B>();
  if (lane < 4) {  // the zero group after the tile's records (never written by the decode)
    constexpr uint32_t NR = batch_rec_elems<B>();
    reinterpret_cast<uint32_t*>(wsm)[NR - 4 + lane] = 0u;
    wsm[(size_t)NR * 4 + NR - 4 + lane] = 0u;
    wsm[(size_t)NR * 5 + NR - 4 + lane] = 0u;
  }
  const uint32_t wpc = blockDim.x >> 5;
  const uint32_t gw = blockIdx.x * wpc + warp;
  const uint32_t nwp = gridDim.x * wpc;
  // blockIdx.y selects the block of 128 queries: the blocks of a batch run as successive waves
  // of one launch, each CTA loading its block's query table once
  const uint32_t blk = a.blk0 + blockIdx.y;
  const uint32_t q0 = blk * kBatchQ;
  const uint32_t nq = min((uint32_t)kBatchQ, a.nq - q0);
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.qtab + (size_t)blk * batch_qtab_words(a.cols));
    uint4* dst = reinterpret_cast<uint4*>(qtb);
    // eight independent loads per thread in flight: the fill is latency-bound otherwise
    const uint32_t n = (uint32_t)(qtab_bytes / 16);
    for (uint32_t i0 = 0; i0 < n; i0 += 8 * blockDim.x) {
      uint4 v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const uint32_t i = i0 + u * blockDim.x + threadIdx.x;
        if (i < n) v[u] = __ldg(src + i);
      }
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const uint32_t i = i0 + u * blockDim.x + threadIdx.x;
        if (i < n) dst[i] = v[u];
      }
    }
  }
  BatchRows<MODE> rows{a, nullptr, {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu},
                       {0x7FFFFFFF, 0x7FFFFFFF, 0x7FFFFFFF, 0x7FFFFFFF}, 0u, lane, q0, nq,
                       MODE == MODE_SAMPLE ? a.keys_out + (size_t)blk * kBatchQ * a.n_sample_rows
                                           : nullptr};
  if constexpr (MODE == MODE_FILTER) {
    if (thr_in_smem) {
      for (uint32_t i = threadIdx.x; i < a.split * kBatchQ; i += blockDim.x) {
        const uint32_t p = i / kBatchQ, q = i % kBatchQ;
        thr_s[i] = q < nq ? a.thr[(size_t)(q0 + q) * a.split + p] : 0xFFFFFFFFu;
      }
      rows.thr_s = thr_s;
    } else if (a.split <= 1) {
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const uint32_t q = 4 * lane + t;
        rows.thr4[t] = q < nq ? a.thr[(size_t)(q0 + q) * a.split] : 0xFFFFFFFFu;
        rows.thr_sc[t] = (int32_t)(rows.thr4[t] ^ 0x80000000u);
      }
    }
  }
  __syncthreads();
  if constexpr (MODE == MODE_SAMPLE) {
    for (uint32_t s = gw; s < a.n_sample_tiles; s += nwp) {
      const uint32_t t = s * a.sample_stride;
      BatchRows<MODE> r2 = rows;
      r2.sample_base = __ldg(a.sample_first + s);
      batch_range<B, SGN, MODE>(a, t, t + 1, r2, qtb, wsm);
    }
  } else {
    const uint64_t n = a.n_tiles;
    const uint32_t tb = (uint32_t)((n * gw) / nwp), te = (uint32_t)((n * (gw + 1)) / nwp);
    batch_range<B, SGN, MODE>(a, tb, te, rows, qtb, wsm);
  }
}

// Sample keys of the batched blocks, [rows][128 queries] per block as the batched sample pass
// writes them, to [query][rows] (the plain layout), so the threshold pass reads each query's keys
// contiguously instead of one 32-byte sector per key.  A CTA moves 32 rows x 128 queries of one
// block (blockIdx.y) through shared memory; both the reads and the writes are coalesced.
constexpr uint32_t kTransposeRows = 32;
__global__ void __launch_bounds__(256) k_keys_transpose(const uint32_t* __restrict__ in,
                                                        uint32_t n_rows, uint32_t nq,
                                                        uint32_t* __restrict__ out) {
  __shared__ uint32_t t[kTransposeRows][kBatchQ + 1];
  const uint32_t blk = blockIdx.y;
  const uint32_t nb = min((uint32_t)kBatchQ, nq - blk * kBatchQ);
  in += (size_t)blk * kBatchQ * n_rows;
  out += (size_t)blk * kBatchQ * n_rows;
  const uint32_t r0 = blockIdx.x * kTransposeRows;
  for (uint32_t i = threadIdx.x; i < kTransposeRows * kBatchQ; i += blockDim.x) {
    const uint32_t rr = i / kBatchQ, q = i % kBatchQ;
    if (r0 + rr < n_rows) t[rr][q] = in[(size_t)(r0 + rr) * kBatchQ + q];
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < kTransposeRows * kBatchQ; i += blockDim.x) {
    const uint32_t q = i / kTransposeRows, rr = i % kTransposeRows;
    if (q < nb && r0 + rr < n_rows) out[(size_t)q * n_rows + r0 + rr] = t[rr][q];
  }
}

// qtab[blk][col][33] words: byte t of word (blk, col, l) = quantised query 128 blk + 4l + t at
// col (0 past nq); word 32 of each column and the padding to a 16-byte slot are zero.  Every
// block of the batch in one launch.
__global__ void k_qtable(const int8_t* __restrict__ q8, uint32_t ld8, uint32_t cols, uint32_t nq,
                         uint32_t* __restrict__ qtab) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nblk = (nq + kBatchQ - 1) / kBatchQ;
  const uint64_t per = batch_qtab_words(cols);
  if (i >= nblk * per) return;
  const uint32_t blk = (uint32_t)(i / per);
  const uint32_t r = (uint32_t)(i % per);
  const uint32_t c = r / kQtabWords, l = r % kQtabWords;
  uint32_t w = 0;
  if (c < cols && l < 32u) {
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const uint32_t q = blk * kBatchQ + 4 * l + t;
      const uint32_t b = q < nq ? (uint32_t)(uint8_t)q8[(size_t)q * ld8 + c] : 0u;
      w |= b << (8 * t);
    }
  }
  qtab[i] = w;
}

}  // namespace dev
}  // namespace aes
