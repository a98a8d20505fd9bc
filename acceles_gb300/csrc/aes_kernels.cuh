// aes_kernels.cuh -- sm_103a candidate pass of the two-stage low-bit Top-K SpMV engine, and the
// helpers the other stages share (the later stages are in aes_select.cuh).
//
// Stages (reference: zhaijiaqi/AccelES):
//   k_cand_plain      the low-bit candidate pass of spmv_ucsr_top_k_main
//                     (spmv_ucsr_top_k_multicore.hpp:195-413; CPU gold spmv_coo_gold_top_k_2,
//                     gold_algorithms.hpp:249-308): streams Ultra-CSR tiles, decodes flags,
//                     10-bit columns and B-bit values in registers, integer row scores
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "aes_qexact.hpp"

namespace aes {
namespace dev {

// warps per CTA of the plain candidate pass: 32 (the 128 KB query table and 32 next-tile buffers
// of 2 KB leave room for the partition thresholds in 227 KB)
__host__ __device__ constexpr int plain_warps(int) { return 32; }
__host__ __device__ constexpr int plain_threads(int B) { return plain_warps(B) * 32; }

enum Mode : int { MODE_FILTER = 0, MODE_SAMPLE = 1, MODE_ALL = 2 };

// status bits per query
constexpr uint32_t ST_OVERFLOW = 1u;  // survivors exceeded the buffer
constexpr uint32_t ST_MISS = 2u;      // fewer survivors than candidates needed
constexpr uint32_t ST_QUERY = 4u;     // query rejected by the quantiser
constexpr uint32_t ST_DEVICE = 8u;    // a bounded wait on the tensor pipe gave up

__host__ __device__ constexpr int packet_elems(int B) { return 511 / (B + 11); }

// order-preserving keys
__device__ __forceinline__ uint32_t key_i32(int32_t s) { return (uint32_t)s ^ 0x80000000u; }
__device__ __forceinline__ uint32_t key_f32(float f) {
  if (f == 0.0f) f = 0.0f;  // -0 == +0 in sort_tuples
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_to_f32(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  return __uint_as_float(u);
}

// compile-time field extraction from the 16 words of a 512-bit packet
template <int POS, int W>
__device__ __forceinline__ uint32_t ufield(const uint32_t (&w)[16]) {
  constexpr int k = POS >> 5, s = POS & 31;
  constexpr uint32_t mask = (W == 32) ? 0xFFFFFFFFu : ((1u << W) - 1u);
  if constexpr (s + W <= 32) {
    return (w[k] >> s) & mask;
  } else {
    return __funnelshift_r(w[k], w[k + 1], s) & mask;
  }
}
template <int POS, int W>
__device__ __forceinline__ int32_t sfield(const uint32_t (&w)[16]) {
  constexpr int k = POS >> 5, s = POS & 31;
  if constexpr (s + W <= 32) {
    return (int32_t)(w[k] << (32 - s - W)) >> (32 - W);
  } else {
    uint32_t x = __funnelshift_r(w[k], w[k + 1], s);
    return (int32_t)(x << (32 - W)) >> (32 - W);
  }
}

struct PlainArgs {
  const uint4* tiles;           // n_tiles * 128 uint4 (tiled layout, see aes_host.hpp)
  const uint32_t* tile_rowbase; // n_tiles + 1
  uint32_t n_tiles, n_rows, cols;
  const int8_t* q8;             // quantised query [cols]
  const float* rowscale;        // per-row scale (unsigned per-row mode) or nullptr
  uint32_t split, slice;        // row partition of a row: min(row / slice, split - 1)
  const uint32_t* thr;          // [split] (MODE_FILTER)
  uint32_t* cnt;                // [split]
  uint2* surv;                  // [split][cap] (key, row)
  uint32_t cap;
  uint32_t* keys_out;           // MODE_SAMPLE: [sample rows]; MODE_ALL: [n_rows]
  const uint32_t* sample_first; // MODE_SAMPLE: owned-row offset per sample tile
  uint32_t sample_stride, n_sample_tiles;
  // MODE_SAMPLE over several queries in one launch: query blockIdx.y reads q8 + y * q8_ld and
  // writes its keys at keys_out + y * keys_ld
  uint32_t q8_ld, keys_ld;
};

constexpr uint32_t kThrSmemMax = 1024;  // thresholds of up to this many partitions in smem

__device__ __forceinline__ uint32_t part_of(uint32_t row, uint32_t split, uint32_t slice) {
  if (split <= 1) return 0;
  uint32_t p = slice ? row / slice : split - 1;
  return p < split - 1 ? p : split - 1;
}

// Where a completed row goes: the survivor buffer (filter), the sample key array, or the
// full key array.
template <int MODE>
struct Emitter {
  const PlainArgs& a;
  const uint32_t* thr_s;  // shared copy of the thresholds (split > 1)
  uint32_t thr0;          // threshold when split == 1
  uint32_t sample_base;   // MODE_SAMPLE: first owned row minus its key index
  // filter with integer keys and one partition: key >= thr0 <=> score >= thr0 ^ 0x80000000
  __device__ __forceinline__ int32_t thr_score() const { return (int32_t)(thr0 ^ 0x80000000u); }
  // a row of the integer filter whose score passed thr_score()
  __device__ __forceinline__ void append_int(uint32_t row, int32_t score) const {
    const uint32_t i = atomicAdd(a.cnt, 1u);
    if (i < a.cap) a.surv[i] = make_uint2(key_i32(score), row);
  }
  // filter with integer keys (no row scales), any number of partitions
  __device__ __forceinline__ bool int_keys() const { return MODE == MODE_FILTER && !a.rowscale; }
  __device__ __forceinline__ uint32_t thr_of(uint32_t p) const {
    return a.split <= 1 ? thr0 : (a.split <= kThrSmemMax ? thr_s[p] : __ldg(a.thr + p));
  }
  // the lowest score bound over the partitions of rows r0 .. r1 (one partition for almost every
  // tile: the partitions are contiguous row ranges)
  __device__ __forceinline__ int32_t score_bound(uint32_t r0, uint32_t r1) const {
    if (a.split <= 1) return thr_score();
    const uint32_t p1 = part_of(r1, a.split, a.slice);
    int32_t b = 0x7FFFFFFF;
    for (uint32_t p = part_of(r0, a.split, a.slice); p <= p1; p++)
      b = min(b, (int32_t)(thr_of(p) ^ 0x80000000u));
    return b;
  }
  // a row whose integer score passed a bound: kept if it passes its own partition's threshold
  __device__ __forceinline__ void append_checked(uint32_t row, int32_t score) const {
    const uint32_t p = part_of(row, a.split, a.slice);
    if (score >= (int32_t)(thr_of(p) ^ 0x80000000u)) {
      const uint32_t i = atomicAdd(a.cnt + p, 1u);
      if (i < a.cap) a.surv[(size_t)p * a.cap + i] = make_uint2(key_i32(score), row);
    }
  }
  __device__ __forceinline__ void operator()(uint32_t row, int32_t score) const {
    uint32_t key;
    if (a.rowscale) key = key_f32(__fmul_rn(__int2float_rn(score), __ldg(a.rowscale + row)));
    else key = key_i32(score);
    if constexpr (MODE == MODE_FILTER) {
      uint32_t p = 0, th = thr0;
      if (a.split > 1) {
        p = part_of(row, a.split, a.slice);
        th = (a.split <= kThrSmemMax) ? thr_s[p] : __ldg(a.thr + p);
      }
      if (key >= th) {
        uint32_t i = atomicAdd(a.cnt + p, 1u);
        if (i < a.cap) a.surv[(size_t)p * a.cap + i] = make_uint2(key, row);
      }
    } else if constexpr (MODE == MODE_SAMPLE) {
      a.keys_out[row - sample_base] = key;
    } else {
      a.keys_out[row] = key;
    }
  }
};

__device__ __forceinline__ void load_tile(const uint4* tiles, uint32_t t, uint32_t lane,
                                          uint32_t (&w)[16]) {
  const uint4* base = tiles + (size_t)t * 128 + lane;
#pragma unroll
  for (int s = 0; s < 4; s++) {
    uint4 v = __ldcs(base + s * 32);
    w[4 * s + 0] = v.x;
    w[4 * s + 1] = v.y;
    w[4 * s + 2] = v.z;
    w[4 * s + 3] = v.w;
  }
}

// bits [POS, POS + 32) of the 512-bit packet held in 16 words
template <int POS>
__device__ __forceinline__ uint32_t window32(const uint32_t (&w)[16]) {
  constexpr int k = POS >> 5, s = POS & 31;
  static_assert(POS >= 0 && POS + 32 <= 512, "window outside the packet");
  if constexpr (s == 0) return w[k];
  else return __funnelshift_r(w[k], w[k + 1], s);
}

// The flag word of a packet: bit j set when entry j starts a row (fpga_utils.hpp:349-384).
template <int B, bool SGN>
struct PacketDecoder {
  static constexpr int P = packet_elems(B);
  using Flags = typename std::conditional<(P <= 32), uint32_t, uint64_t>::type;

  __device__ __forceinline__ static Flags flags(const uint32_t (&w)[16]) {
    if constexpr (P <= 32) {
      return w[0] & ((P == 32) ? 0xFFFFFFFFu : ((1u << P) - 1u));
    } else {
      return (uint64_t)w[0] | ((uint64_t)(w[1] & ((1u << (P - 32)) - 1u)) << 32);
    }
  }
};

// Per-lane decode of one packet in spans.  Element j: 10-bit column at bit P + 10j, B-bit value
// at bit 11P + Bj (fpga_utils.hpp:349-384).  A group of four entries is one dp4a of its four
// values (unpacked to bytes in element order) with the four query bytes.  A row that starts and
// ends inside the packet is scored while the groups are decoded: the running sum at a flag is
// the sum before its span plus a dp4a of the bytes before it.  Nothing is staged in shared
// memory; only the row closed by a lane's first flag needs the running sums of the lanes before
// it, which the warp scan gives after the decode.
struct Rows8 {
  int32_t S;       // running sum of the packet so far
  uint32_t first;  // running sum before the first flagged entry
  uint32_t prev;   // running sum before the last flagged entry so far
  uint32_t row;    // row closed by the next flag
  bool seen;       // a flag was met
};

template <int B, bool SGN>
struct PacketSpans {
  static constexpr int P = packet_elems(B);
  static constexpr int NG = (P + 3) / 4;
  using Flags = typename PacketDecoder<B, SGN>::Flags;

  // q[col_J] from the lane-replicated 32-bit table qt[col][32]: lane l reads bank l whatever the
  // columns, so a gather is one wavefront.  The column window starts 7 bits early so
  // (col << 7), the row offset of col in the table, lands at bits 7..16.
  template <int J>
  __device__ __forceinline__ static uint32_t qval(const uint32_t (&w)[16], const char* qtb,
                                                  uint32_t lane4) {
    const uint32_t y = window32<P + 10 * J - 7>(w);
    return *reinterpret_cast<const uint32_t*>(qtb + ((y & 0x1FF80u) | lane4));
  }

  __device__ __forceinline__ static int32_t dot4(uint32_t v4, uint32_t q4, int32_t c) {
    return SGN ? __dp4a((int)v4, (int)q4, c) : (int32_t)__dp4a(v4, q4, (unsigned)c);
  }

  // bits [POS, POS + 32) of the packet, or, near its end, the 32 bits ending at bit 512 shifted
  // down so that bit POS comes first (the bits above the packet's end read as zero)
  template <int POS>
  __device__ __forceinline__ static uint32_t field32(const uint32_t (&w)[16]) {
    if constexpr (POS + 32 <= 512) return window32<POS>(w);
    else return window32<480>(w) >> (POS - 480);
  }

  // Scores of signed 6-bit packets come out four times too large: their values sit at bits 2-7
  // of each byte (unpack), where the byte's sign is the value's, so no sign extension is needed;
  // sums of them are exact multiples of four, shifted back where a row's score is emitted.
  static constexpr int kScoreShift = (B == 6 && SGN) ? 2 : 0;

  // the four B-bit values at the bottom of x as bytes in element order (sign-extended when SGN;
  // signed 6-bit: four times each value)
  __device__ __forceinline__ static uint32_t unpack(uint32_t x) {
    if constexpr (B == 8) {
      return x;
    } else if constexpr (B == 4) {
      const uint32_t z = __byte_perm(x, 0u, 0x4140);  // entries 0,1 | 0 | entries 2,3 | 0
      uint32_t v = (z | (z * 16u)) & 0x0F0F0F0Fu;
      if constexpr (SGN) v |= (v & 0x08080808u) * 0x1Eu;  // bit 3 -> bits 4..7 of each byte
      return v;
    } else if constexpr (SGN) {
      static_assert(B == 6, "bit width");
      // bits 0-11 of h are values 0 and 1, bits 16-27 values 2 and 3 (bits 12-15 and 28-31 are
      // never selected below); value k then goes to bits 8k + 2 .. 8k + 7
      const uint32_t x16 = x * 16u;
      const uint32_t h = (x & 0xFFFu) | (x16 & 0xFFFFF000u);
      return ((h * 4u) & 0x00FC00FCu) | ((h * 16u) & 0xFC00FC00u);
    } else {
      static_assert(B == 6, "bit width");
      const uint32_t h = (x & 0xFFFu) | ((x * 16u) & 0x0FFF0000u);      // 12-bit halves
      return (h & 0x003F003Fu) | ((h * 4u) & 0x3F003F00u);              // 6-bit bytes
    }
  }

  // q0..q3 of group G packed into one word, and its four values
  template <int G>
  __device__ __forceinline__ static void load_group(const uint32_t (&w)[16], const char* qtb,
                                                    uint32_t lane4, uint32_t& q4, uint32_t& v4) {
    constexpr int J = 4 * G;
    constexpr int n = (P - J) < 4 ? (P - J) : 4;  // entries in this group
    // table entries are zero-extended bytes, so multiply-adds place them (FMA pipe, leaving
    // the integer ALU pipe to the field extraction)
    q4 = qval<J>(w, qtb, lane4);
    if constexpr (n > 1) q4 += qval<(n > 1 ? J + 1 : J)>(w, qtb, lane4) * 0x100u;
    if constexpr (n > 2) q4 += qval<(n > 2 ? J + 2 : J)>(w, qtb, lane4) * 0x10000u;
    if constexpr (n > 3) q4 += qval<(n > 3 ? J + 3 : J)>(w, qtb, lane4) * 0x1000000u;
    v4 = unpack(field32<11 * P + B * J>(w));
    if constexpr (n < 4) v4 &= (1u << (8 * n)) - 1u;
  }

  // The running sum at flag j of the span starting at group G (NGR groups): the sum before the
  // span plus the dp4a of the bytes before j, masked out of the packed values.
  template <int G, int NGR>
  __device__ __forceinline__ static uint32_t span_prefix(int j, int32_t Sa, uint32_t qa,
                                                         uint32_t va, uint32_t qb, uint32_t vb,
                                                         uint32_t qc, uint32_t vc) {
    const uint64_t m = ~(~0ull << (8 * (j & 7)));  // bytes before entry j (j < 8)
    if constexpr (NGR == 2) {
      return (uint32_t)dot4(vb & (uint32_t)(m >> 32), qb, dot4(va & (uint32_t)m, qa, Sa));
    } else {
      const bool lo = j < 8;
      const uint32_t ma = lo ? (uint32_t)m : 0xFFFFFFFFu;
      const uint32_t mb = lo ? (uint32_t)(m >> 32) : 0xFFFFFFFFu;
      const uint32_t mc = lo ? 0u : ~(0xFFFFFFFFu << (8 * ((j - 8) & 3)));
      const int32_t x = dot4(vb & mb, qb, dot4(va & ma, qa, Sa));
      return (uint32_t)dot4(vc & mc, qc, x);
    }
  }

  // Spans of two groups (eight entries); the last takes a short tail group as a third
  // (B = 8: 8/8/10 entries, B = 6: 8/8/8/6, B = 4: 8/8/8/10).
  template <int G>
  __host__ __device__ static constexpr int span_groups() { return (G + 3 == NG) ? 3 : 2; }
  // flag bits of the span starting at group G, in place
  template <int G>
  __host__ __device__ static constexpr uint64_t span_bits() {
    return ((P - 4 * G) < 4 * span_groups<G>() ? ((1ull << (P - 4 * G)) - 1ull)
                                               : ((1ull << (4 * span_groups<G>())) - 1ull))
           << (4 * G);
  }
  // true when some span from group G on holds two or more flags (a row shorter than a span)
  template <int G = 0>
  __device__ __forceinline__ static bool two_in_a_span(Flags F) {
    if constexpr (G >= NG) {
      return false;
    } else {
      const Flags f = F & (Flags)span_bits<G>();
      return (f & (f - 1)) != 0 || two_in_a_span<G + span_groups<G>()>(F);
    }
  }

  // Decode the span starting at group G and score the rows closed by its flags: each closed row
  // goes to on_row(valid, row, score) (INNER: not on the closing tile).  The lowest flag of the
  // span is handled without a branch; further flags (multi: some lane of the warp has them) in
  // a loop.
  template <int G, bool INNER, class OnRow>
  __device__ __forceinline__ static void span(const uint32_t (&w)[16], const char* qtb,
                                              uint32_t lane4, Flags F, bool multi, Rows8& s,
                                              const OnRow& on_row) {
    if constexpr (G < NG) {
      constexpr int NGR = span_groups<G>();
      static_assert(G + NGR <= NG, "span layout");
      uint32_t qa, va, qb, vb, qc = 0u, vc = 0u;
      load_group<G>(w, qtb, lane4, qa, va);
      load_group<G + 1>(w, qtb, lane4, qb, vb);
      if constexpr (NGR == 3) load_group<(NGR == 3 ? G + 2 : G)>(w, qtb, lane4, qc, vc);
      const int32_t Sa = s.S;
      s.S = dot4(vb, qb, dot4(va, qa, Sa));
      if constexpr (NGR == 3) s.S = dot4(vc, qc, s.S);
      const uint32_t fP = (uint32_t)((F & (Flags)span_bits<G>()) >> (4 * G));
      const bool has = fP != 0;
      const uint32_t Pj = span_prefix<G, NGR>(__ffs(fP) - 1, Sa, qa, va, qb, vb, qc, vc);
      if constexpr (INNER) on_row(has && s.seen, s.row, (int32_t)(Pj - s.prev));
      s.first = (has && !s.seen) ? Pj : s.first;
      s.prev = has ? Pj : s.prev;
      s.row += has ? 1u : 0u;
      s.seen = s.seen || has;
      if (multi) {
        uint32_t rest = fP & (fP - 1u);
        while (rest) {
          const int j = __ffs(rest) - 1;
          rest &= rest - 1u;
          const uint32_t Pk = span_prefix<G, NGR>(j, Sa, qa, va, qb, vb, qc, vc);
          if constexpr (INNER) on_row(true, s.row, (int32_t)(Pk - s.prev));
          s.prev = Pk;
          s.row++;
        }
      }
      span<G + NGR, INNER>(w, qtb, lane4, F, multi, s, on_row);
    }
  }
};

__device__ __forceinline__ int ffs_flags(uint32_t f) { return __ffs(f) - 1; }
__device__ __forceinline__ int ffs_flags(uint64_t f) { return __ffsll((long long)f) - 1; }
__device__ __forceinline__ int fls_flags(uint32_t f) { return 31 - __clz(f); }
__device__ __forceinline__ int fls_flags(uint64_t f) { return 63 - __clzll((long long)f); }
__device__ __forceinline__ uint32_t popc_flags(uint32_t f) { return __popc(f); }
__device__ __forceinline__ uint32_t popc_flags(uint64_t f) { return __popcll(f); }

// inclusive warp sum; shfl.up's own predicate (source lane in range) guards each add
__device__ __forceinline__ uint32_t warp_incl_sum(uint32_t v, uint32_t lane) {
  (void)lane;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    asm("{\n\t.reg .b32 t;\n\t.reg .pred p;\n\t"
        "shfl.sync.up.b32 t|p, %0, %1, 0, 0xffffffff;\n\t"
        "@p add.u32 %0, %0, t;\n\t}"
        : "+r"(v)
        : "r"(d));
  }
  return v;
}

struct RangeState {
  bool open_owned;  // the row open at the current position started inside the range
  uint32_t startG;  // running sum before the open row's first entry
  uint32_t carryG;  // running sum before the current tile
};

// How a plain pass emits rows: any emitter, or the filter with integer keys (no row scales) and
// one partition, or with several partitions.
enum EmitKind : int { EMIT_ANY = 0, EMIT_INT_ONE = 1, EMIT_INT_PARTS = 2 };

// The partition of a warp's current tile, followed across tiles without a division.
struct PartTrack {
  uint32_t p;    // partition of the tile's first row
  uint32_t end;  // first row of partition p + 1 (0xFFFFFFFF: p is the last)
  int32_t ts;    // score bound of partition p
};

// One tile of a warp's range.  Returns true once the range is complete.
// KIND EMIT_INT_*: a compare per row against the score bound of the partition of the tile's rows
// (the lowest over its partitions when it straddles some), and the exact check and survivor
// append only on a hit.  CLOSING: a tile at or past the range's end, where only the first flag
// matters.
template <int B, bool SGN, int MODE, int KIND, bool CLOSING>
__device__ __forceinline__ bool tile_step(const PlainArgs& a, uint32_t t,
                                           const uint32_t (&w)[16], uint32_t rowbase,
                                           RangeState& st, const Emitter<MODE>& emit,
                                           const char* qtb, PartTrack& pt) {
  using D = PacketSpans<B, SGN>;
  using Flags = typename D::Flags;
  const uint32_t lane = threadIdx.x & 31u;
  if constexpr (CLOSING) {
    if (t >= a.n_tiles) {  // the end of the matrix closes the last row
      if (st.open_owned && lane == 0)
        emit(a.n_rows - 1, (int32_t)(st.carryG - st.startG) >> D::kScoreShift);
      return true;
    }
  }
  const Flags F = PacketDecoder<B, SGN>::flags(w);
  const uint32_t has_mask = __ballot_sync(0xFFFFFFFFu, F != 0);
  uint32_t rbase = rowbase;  // row closed by this lane's first flag
  int32_t ts = 0;            // EMIT_INT_*: score bound of the rows this tile closes
  if constexpr (!CLOSING) {
    const uint32_t nf = popc_flags(F);
    const uint32_t incl = warp_incl_sum(nf, lane);
    rbase += incl - nf;
    if constexpr (KIND == EMIT_INT_ONE) ts = emit.thr_score();
    if constexpr (KIND == EMIT_INT_PARTS) {
      const uint32_t r1 = rowbase + __shfl_sync(0xFFFFFFFFu, incl, 31);
      while (rowbase >= pt.end) {  // the tile starts in a later partition
        pt.p++;
        pt.end = (pt.p + 1 >= a.split) ? 0xFFFFFFFFu : pt.end + a.slice;
        pt.ts = (int32_t)(emit.thr_of(pt.p) ^ 0x80000000u);
      }
      ts = r1 < pt.end ? pt.ts : emit.score_bound(rowbase, r1);
    }
  }
  auto on_row = [&](bool valid, uint32_t row, int32_t sc4) {
    const int32_t sc = sc4 >> D::kScoreShift;
    if constexpr (KIND == EMIT_INT_ONE) {
      if (valid && sc >= ts) emit.append_int(row, sc);
    } else if constexpr (KIND == EMIT_INT_PARTS) {
      if (valid && sc >= ts) emit.append_checked(row, sc);
    } else {
      if (valid) emit(row, sc);
    }
  };
  const bool multi = !CLOSING && __any_sync(0xFFFFFFFFu, D::two_in_a_span(F));
  Rows8 s{0, 0u, 0u, rbase, false};
  D::template span<0, !CLOSING>(w, qtb, lane << 2, F, multi, s, on_row);
  const uint32_t total = (uint32_t)s.S;
  const uint32_t incl = warp_incl_sum(total, lane);
  const uint32_t LB = st.carryG + incl - total;  // running sum before this packet
  const uint32_t tileSum = __shfl_sync(0xFFFFFFFFu, incl, 31);
  if constexpr (CLOSING) {
    if (has_mask == 0) {
      st.carryG += tileSum;
      return false;
    }
    if (lane == (uint32_t)(__ffs(has_mask) - 1) && st.open_owned)
      emit(rowbase, (int32_t)(LB + s.first - st.startG) >> D::kScoreShift);
    return true;
  } else {
    // the row closed by a lane's first flag started at the last flag of the lanes before it,
    // or before the tile
    const uint32_t lastGb = LB + s.prev;
    const uint32_t left = has_mask & ((1u << lane) - 1u);
    const uint32_t inhG = __shfl_sync(0xFFFFFFFFu, lastGb, left ? (31 - __clz(left)) : 0u);
    const uint32_t prevG = left ? inhG : st.startG;
    on_row(F && (left || st.open_owned), rbase, (int32_t)(LB + s.first - prevG));
    if (has_mask) {
      st.startG = __shfl_sync(0xFFFFFFFFu, lastGb, 31 - __clz(has_mask));
      st.open_owned = true;
    }
    st.carryG += tileSum;
    return false;
  }
}

// One warp streams tiles [tb, te) and owns every row whose first entry lies in them; the row
// still open at te is finished by reading on until the next row flag.  The next tile is copied
// into the warp's shared buffer with cp.async while the current one is scored; each lane copies,
// and later reads back, only its own 64 bytes, so no synchronisation between lanes is needed.
// Tiles up to te (the first closing tile) are fetched one ahead; tiles past te only when the open
// row runs on through the closing tile.
template <int B, bool SGN, int MODE, int KIND>
__device__ void cand_range(const PlainArgs& a, uint32_t tb, uint32_t te,
                           const Emitter<MODE>& emit, const char* qtb, uint4* stg) {
  const uint32_t lane = threadIdx.x & 31u;
  if (tb >= te) return;
  RangeState st{tb == 0, 0u, 0u};  // row 0 starts at entry 0 without a flag
  PartTrack pt{0u, 0xFFFFFFFFu, 0};
  if constexpr (KIND == EMIT_INT_PARTS) {
    const uint32_t r0 = __ldg(a.tile_rowbase + tb);
    pt.p = part_of(r0, a.split, a.slice);
    pt.end = (pt.p + 1 >= a.split || a.slice == 0) ? 0xFFFFFFFFu : (pt.p + 1) * a.slice;
    pt.ts = (int32_t)(emit.thr_of(pt.p) ^ 0x80000000u);
  }
  uint32_t w[16];
  uint32_t rn = 0;
  auto fetch = [&](uint32_t t) {
    if (t < a.n_tiles) {
      const uint4* src = a.tiles + (size_t)t * 128 + lane;
#pragma unroll
      for (int s = 0; s < 4; s++) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(stg + s * 32 + lane);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src + s * 32)
                     : "memory");
      }
      rn = __ldg(a.tile_rowbase + t);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  fetch(tb);
  for (uint32_t t = tb;; t++) {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const uint4 v = stg[s * 32 + lane];
      w[4 * s + 0] = v.x;
      w[4 * s + 1] = v.y;
      w[4 * s + 2] = v.z;
      w[4 * s + 3] = v.w;
    }
    const uint32_t r = rn;
    if (t + 1 <= te) fetch(t + 1);
    if (t < te) {  // te <= n_tiles
      tile_step<B, SGN, MODE, KIND, false>(a, t, w, r, st, emit, qtb, pt);
    } else if (tile_step<B, SGN, MODE, KIND, true>(a, t, w, r, st, emit, qtb, pt)) {
      return;
    }
    if (t + 1 > te) fetch(t + 1);
  }
}

// query table bytes per column: 32 lane copies of 32 bits (one wavefront per gather)
constexpr size_t kPlainTableBytesPerCol = 128;
constexpr size_t kPlainTileBuf = 2048;  // per warp: the next 32-packet tile

// dynamic shared memory of the plain pass: lane-replicated query table, per-warp next-tile
// buffer, thresholds of up to kThrSmemMax partitions
__host__ inline size_t plain_smem_bytes(int B, uint32_t cols, uint32_t split) {
  return (size_t)cols * kPlainTableBytesPerCol + (size_t)plain_warps(B) * kPlainTileBuf +
         (split > 1 && split <= kThrSmemMax ? split * 4ull : 0ull);
}

template <int B, bool SGN, int MODE>
__global__ void __launch_bounds__(plain_threads(B), 1) k_cand_plain(PlainArgs a) {
  constexpr int W = plain_warps(B);
  extern __shared__ __align__(16) unsigned char smem[];
  // the warp index through a shuffle from lane 0, so the range bounds and every branch on them
  // are known to be warp-uniform
  const uint32_t warp = __shfl_sync(0xFFFFFFFFu, threadIdx.x >> 5, 0);
  const char* qtb = reinterpret_cast<const char*>(smem);  // qt[cols][32 lanes]
  unsigned char* after = smem + (size_t)a.cols * kPlainTableBytesPerCol;
  uint4* stg = reinterpret_cast<uint4*>(after) + (size_t)warp * (kPlainTileBuf / 16);
  uint32_t* thr_s = reinterpret_cast<uint32_t*>(after + W * kPlainTileBuf);
  // replicate the query once per lane; the bytes are staged through the (not yet used) area
  // after the table so the fill needs one global round trip
  int8_t* qstage = reinterpret_cast<int8_t*>(after);
  const int8_t* q8 = a.q8 + (size_t)blockIdx.y * a.q8_ld;
  for (uint32_t i = threadIdx.x; i < a.cols; i += blockDim.x) qstage[i] = q8[i];
  __syncthreads();
  {
    uint4* qt = reinterpret_cast<uint4*>(smem);  // four lane copies per store
    for (uint32_t i = threadIdx.x; i < a.cols * 8u; i += blockDim.x) {
      const uint32_t v = (uint8_t)qstage[i >> 3];  // the byte dp4a reads (signed or not)
      qt[i] = make_uint4(v, v, v, v);
    }
  }
  __syncthreads();
  uint32_t thr0 = 0;
  if constexpr (MODE == MODE_FILTER) {
    if (a.split > 1 && a.split <= kThrSmemMax)
      for (uint32_t i = threadIdx.x; i < a.split; i += blockDim.x) thr_s[i] = a.thr[i];
    thr0 = a.thr[0];
  }
  __syncthreads();
  const uint32_t gw = blockIdx.x * W + warp;
  const uint32_t nw = gridDim.x * W;
  if constexpr (MODE == MODE_SAMPLE) {
    for (uint32_t s = gw; s < a.n_sample_tiles; s += nw) {
      const uint32_t t = s * a.sample_stride;
      // keys of query y land keys_ld further on: the index row - base wraps to that offset
      Emitter<MODE> em{a, thr_s, thr0, __ldg(a.sample_first + s) - blockIdx.y * a.keys_ld};
      cand_range<B, SGN, MODE, EMIT_ANY>(a, t, t + 1, em, qtb, stg);
    }
  } else {
    const uint64_t n = a.n_tiles;
    const uint32_t tb = (uint32_t)((n * gw) / nw), te = (uint32_t)((n * (gw + 1)) / nw);
    Emitter<MODE> em{a, thr_s, thr0, 0u};
    if constexpr (MODE == MODE_FILTER) {
      if (em.int_keys()) {
        if (a.split <= 1) cand_range<B, SGN, MODE, EMIT_INT_ONE>(a, tb, te, em, qtb, stg);
        else cand_range<B, SGN, MODE, EMIT_INT_PARTS>(a, tb, te, em, qtb, stg);
        return;
      }
    }
    cand_range<B, SGN, MODE, EMIT_ANY>(a, tb, te, em, qtb, stg);
  }
}

}  // namespace dev
}  // namespace aes
