// aes_host.cpp -- host-side data preparation: FP32 CSR, quantisers, empty-row rule, Ultra-CSR
// packing in the tiled device layout, and the seeded synthetic matrix generator.
//
// Reference anchors (zhaijiaqi/AccelES):
//   quantify_matrix           src/resources/python/quantify/quantify_util.py:8-28
//   check_empty_rows          src/resources/python/quantify/quantify_util.py:440-445
//   partitioning              src/resources/python/quantify/quantify_util.py:185-189
//                             (host_spmv_ucsr.cpp:204-214 agrees when rows % 32 == 0)
//   Q_packet_coo(_partition)  src/fpga/src/host_spmv_ucsr.cpp:278-319, :388-425
//   Q_write_block_x/y/val     src/fpga/src/ip/fpga_utils.hpp:438-503
#include "aes_host.hpp"
#include "aes_tc_layout.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <thread>

namespace aes {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
const char* last_error_cstr() { return g_last_error.c_str(); }

void parallel_for(uint64_t n, uint64_t grain, const std::function<void(uint64_t, uint64_t)>& fn) {
  if (n == 0) return;
  unsigned hw = std::thread::hardware_concurrency();
  if (hw == 0) hw = 1;
  uint64_t nt = std::min<uint64_t>(hw, (n + grain - 1) / grain);
  if (nt <= 1) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  uint64_t chunk = (n + nt - 1) / nt;
  for (uint64_t t = 0; t < nt; t++) {
    uint64_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([&fn, b, e] { fn(b, e); });
  }
  for (auto& x : th) x.join();
}

int check_csr(const uint64_t* ptr, const uint32_t* col, uint32_t rows, uint32_t cols) {
  if (ptr[0] != 0) return fail(AES_ERR_INVALID, "csr ptr[0] must be 0");
  for (uint32_t r = 0; r < rows; r++) {
    if (ptr[r + 1] < ptr[r]) return fail(AES_ERR_INVALID, "csr ptr not monotone");
    for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) {
      if (col[e] >= cols) return fail(AES_ERR_INVALID, "column index out of range");
      if (e > ptr[r] && col[e] < col[e - 1])
        return fail(AES_ERR_INVALID, "csr columns not sorted within a row");
    }
  }
  return AES_OK;
}

int coo_to_csr(const uint32_t* row, const uint32_t* col, const float* val, uint32_t rows,
               uint32_t cols, uint64_t nnz, HostCSR* out, const int8_t* qval) {
  out->rows = rows;
  out->cols = cols;
  out->ptr.assign((size_t)rows + 1, 0);
  for (uint64_t i = 0; i < nnz; i++) {
    if (row[i] >= rows) return fail(AES_ERR_INVALID, "row index out of range");
    if (col[i] >= cols) return fail(AES_ERR_INVALID, "column index out of range");
    out->ptr[row[i] + 1]++;
  }
  for (uint32_t r = 0; r < rows; r++) out->ptr[r + 1] += out->ptr[r];
  out->col.resize(nnz);
  out->val.resize(val ? nnz : 0);
  out->qv.resize(qval ? nnz : 0);
  std::vector<uint64_t> pos(out->ptr.begin(), out->ptr.end() - 1);
  for (uint64_t i = 0; i < nnz; i++) {  // stable counting sort by row
    uint64_t d = pos[row[i]]++;
    out->col[d] = col[i];
    if (val) out->val[d] = val[i];
    if (qval) out->qv[d] = qval[i];
  }
  // stable sort by column inside each row (readMtx sorts tuples by (row, col), utils.hpp:331)
  parallel_for(rows, 4096, [&](uint64_t b, uint64_t e) {
    std::vector<uint64_t> order;
    std::vector<uint32_t> tc;
    std::vector<float> tv;
    std::vector<int8_t> tq;
    for (uint64_t r = b; r < e; r++) {
      uint64_t s = out->ptr[r], t = out->ptr[r + 1];
      bool sorted = true;
      for (uint64_t k = s + 1; k < t; k++)
        if (out->col[k] < out->col[k - 1]) { sorted = false; break; }
      if (sorted) continue;
      order.resize(t - s);
      for (uint64_t k = s; k < t; k++) order[k - s] = k;
      std::stable_sort(order.begin(), order.end(),
                       [&](uint64_t x, uint64_t y) { return out->col[x] < out->col[y]; });
      tc.resize(t - s);
      for (uint64_t k = 0; k < t - s; k++) tc[k] = out->col[order[k]];
      std::copy(tc.begin(), tc.end(), out->col.begin() + s);
      if (val) {
        tv.resize(t - s);
        for (uint64_t k = 0; k < t - s; k++) tv[k] = out->val[order[k]];
        std::copy(tv.begin(), tv.end(), out->val.begin() + s);
      }
      if (qval) {
        tq.resize(t - s);
        for (uint64_t k = 0; k < t - s; k++) tq[k] = out->qv[order[k]];
        std::copy(tq.begin(), tq.end(), out->qv.begin() + s);
      }
    }
  });
  return AES_OK;
}

// ---------------------------------------------------------------------------------------------
// quantisers (float64 arithmetic of quantify_util.py, round half to even)
// ---------------------------------------------------------------------------------------------

static inline int32_t q_sym(double v, double m, int bits) {
  int32_t M = ((1 << bits) - 1) / 2;
  if (m == 0.0) return 0;
  double y = (double)M * (v / m);
  int32_t q = (int32_t)std::nearbyint(y);
  return std::min(std::max(q, -M - 1), M);
}

static inline int32_t q_uns(double v, double m, int bits) {
  int32_t M = (1 << bits) - 1;
  if (m == 0.0) return 0;
  double y = (double)M * (v / m);
  int32_t q = (int32_t)std::nearbyint(y);
  return std::min(std::max(q, 0), M);
}

static inline uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// 512-bit packet under construction; bit i of the packet is bit (i & 63) of word i >> 6, i.e.
// byte i >> 3, bit i & 7 in little-endian memory (ap_uint<512>::range, fpga_utils.hpp:438-503).
struct Bits512 {
  uint64_t w[8];
  void clear() { std::memset(w, 0, sizeof(w)); }
  void put(int pos, int width, uint64_t v) {
    v &= (width == 64) ? ~0ull : ((1ull << width) - 1);
    int k = pos >> 6, s = pos & 63;
    w[k] |= v << s;
    if (s + width > 64) w[k + 1] |= v >> (64 - s);
  }
};

// Tensor-core layout of a 4-bit matrix (PackedMatrix::tc_*).  Left empty when a row holds a
// column twice (the dense tile would keep one of the two values) or nnz needs 64-bit offsets.
static void build_tc_layout(const std::vector<uint64_t>& qptr, const std::vector<uint16_t>& qcol,
                            const std::vector<int8_t>& qval, PackedMatrix* out) {
  const uint32_t rows = out->rows;
  const uint64_t qnnz = qptr[rows];
  if (qnnz > 0xFFFFFFFFull) return;
  const uint32_t nch = tc_nchunks(out->cols);
  const uint64_t nt = ((uint64_t)rows + kTcRows - 1) / kTcRows;
  std::vector<uint32_t> cnt(nt * nch + 1, 0);
  std::vector<char> dup(nt, 0);
  parallel_for(nt, 64, [&](uint64_t b, uint64_t e) {
    for (uint64_t t = b; t < e; t++) {
      const uint64_t r1 = std::min<uint64_t>(rows, (t + 1) * kTcRows);
      for (uint64_t r = t * kTcRows; r < r1; r++) {
        std::vector<uint64_t> seen;
        for (uint64_t i = qptr[r]; i < qptr[r + 1]; i++) {
          cnt[t * nch + qcol[i] / kTcChunkK]++;
          // columns are in order within a row unless the input holds duplicates
          if (i > qptr[r] && qcol[i] <= qcol[i - 1]) {
            if (seen.empty()) {
              seen.assign(16, 0);
              for (uint64_t j = qptr[r]; j < i; j++) seen[qcol[j] >> 6] |= 1ull << (qcol[j] & 63);
            }
            if (seen[qcol[i] >> 6] >> (qcol[i] & 63) & 1) dup[t] = 1;
          }
          if (!seen.empty()) seen[qcol[i] >> 6] |= 1ull << (qcol[i] & 63);
        }
      }
    }
  });
  for (uint64_t t = 0; t < nt; t++)
    if (dup[t]) return;
  out->tc_ptr.assign(nt * nch + 1, 0);
  for (uint64_t j = 0; j < nt * nch; j++) out->tc_ptr[j + 1] = out->tc_ptr[j] + cnt[j];
  // Within a (tile, chunk) the order is free: entries go round-robin over the 32 shared-memory
  // banks their bytes fall in (bank = offset / 4 % 32), so the 32 consecutive entries one warp
  // writes with one store instruction hit distinct banks as long as every bank has entries left.
  out->tc_ent.assign(qnnz, 0);
  parallel_for(nt, 64, [&](uint64_t b, uint64_t e) {
    std::vector<std::vector<uint32_t>> chunk(nch);
    std::vector<uint32_t> bank_n(32), keyed;
    for (uint64_t t = b; t < e; t++) {
      for (auto& v : chunk) v.clear();
      const uint64_t r1 = std::min<uint64_t>(rows, (t + 1) * kTcRows);
      for (uint64_t r = t * kTcRows; r < r1; r++) {
        for (uint64_t i = qptr[r]; i < qptr[r + 1]; i++) {
          const uint32_t c = qcol[i] / kTcChunkK, k = qcol[i] % kTcChunkK;
          chunk[c].push_back((tc_off((uint32_t)(r - t * kTcRows), k) << 16) |
                             (uint32_t)e4m3_small((int)qval[i]));
        }
      }
      for (uint32_t c = 0; c < nch; c++) {
        // key = (rank among the entries of its bank) * 32 + bank; ascending keys go round-robin
        std::fill(bank_n.begin(), bank_n.end(), 0u);
        keyed.clear();
        for (size_t j = 0; j < chunk[c].size(); j++) {
          const uint32_t bank = (chunk[c][j] >> 18) & 31u;
          keyed.push_back(bank_n[bank]++ * 32u + bank);
        }
        std::vector<uint32_t> order(chunk[c].size());
        for (size_t j = 0; j < order.size(); j++) order[j] = (uint32_t)j;
        std::sort(order.begin(), order.end(),
                  [&](uint32_t x, uint32_t y) { return keyed[x] < keyed[y]; });
        uint32_t* dst = out->tc_ent.data() + out->tc_ptr[t * nch + c];
        for (size_t j = 0; j < order.size(); j++) dst[j] = chunk[c][order[j]];
      }
    }
  });
  out->tc_nch = nch;
}

int quantize_and_pack(const HostCSR& m, const aes_params& p, PackedMatrix* out) {
  const uint32_t rows = m.rows;
  const int bits = (int)p.bits;
  const int P = packet_elems(bits);
  const uint64_t nnz = m.ptr[rows];
  out->rows = rows;
  out->cols = m.cols;
  out->bits = (uint32_t)bits;
  out->quant = p.quant;
  out->P = (uint32_t)P;

  const bool preq = m.prequantized;
  if (preq && p.quant != AES_QUANT_SYM_GLOBAL)
    return fail(AES_ERR_UNSUPPORTED, "pre-quantised matrices take the symmetric B-bit values");
  if (preq) {
    const int32_t lo = -(1 << (bits - 1)), hi = (1 << (bits - 1)) - 1;
    for (uint64_t k = 0; k < nnz; k++)
      if (m.qv[k] < lo || m.qv[k] > hi)
        return fail(AES_ERR_INVALID, "pre-quantised value outside the signed B-bit range");
  }

  // ---- scale ---------------------------------------------------------------------------------
  double gmax = 0.0;
  bool negative = false;
  if (!preq) {
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<double> part(nt, 0.0);
    std::vector<char> neg(nt, 0);
    std::vector<std::thread> th;
    uint64_t chunk = (nnz + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++) {
      th.emplace_back([&, t] {
        uint64_t b = (uint64_t)t * chunk, e = std::min(nnz, b + chunk);
        double mx = 0.0;
        char ng = 0;
        for (uint64_t i = b; i < e; i++) {
          double a = std::fabs((double)m.val[i]);
          if (a > mx) mx = a;
          if (m.val[i] < 0.0f) ng = 1;
        }
        part[t] = mx;
        neg[t] = ng;
      });
    }
    for (auto& x : th) x.join();
    for (unsigned t = 0; t < nt; t++) {
      gmax = std::max(gmax, part[t]);
      negative |= (neg[t] != 0);
    }
  }
  if (p.quant != AES_QUANT_SYM_GLOBAL && negative)
    return fail(AES_ERR_INVALID, "unsigned quantiser needs non-negative matrix values");

  const bool per_row = (p.quant == AES_QUANT_UNSIGNED_ROW);
  const bool is_signed = (p.quant == AES_QUANT_SYM_GLOBAL);
  if (per_row) out->rowscale.assign(rows, 0.0f);
  const double Mrow = (double)((1 << bits) - 1);

  // ---- pass 1: kept entries per row ------------------------------------------------------------
  std::vector<uint64_t> qptr((size_t)rows + 1, 0);
  parallel_for(rows, 1 << 14, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; r++) {
      uint64_t s = m.ptr[r], t = m.ptr[r + 1];
      if (preq) {  // every given entry is kept
        qptr[r + 1] = t > s ? t - s : 1;
        continue;
      }
      double sc = gmax;
      if (per_row) {
        sc = 0.0;
        for (uint64_t k = s; k < t; k++) sc = std::max(sc, (double)m.val[k]);
        out->rowscale[r] = (float)(sc / Mrow);
      }
      uint64_t cnt = 0;
      for (uint64_t k = s; k < t; k++) {
        int32_t q = is_signed ? q_sym(m.val[k], sc, bits) : q_uns(m.val[k], sc, bits);
        cnt += (q != 0);
      }
      qptr[r + 1] = cnt ? cnt : 1;  // a row left empty gets one entry
    }
  });
  for (uint32_t r = 0; r < rows; r++) qptr[r + 1] += qptr[r];
  const uint64_t qnnz = qptr[rows];
  out->qnnz = qnnz;
  std::vector<uint16_t> qcol(qnnz);
  std::vector<int8_t> qval(qnnz);  // B <= 8 fits; unsigned values are stored as their low byte
  parallel_for(rows, 1 << 14, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; r++) {
      uint64_t s = m.ptr[r], t = m.ptr[r + 1];
      if (preq) {
        uint64_t o = qptr[r];
        for (uint64_t k = s; k < t; k++, o++) {
          qcol[o] = (uint16_t)m.col[k];
          qval[o] = m.qv[k];
        }
        if (t == s) {  // a row without entries: one zero entry keeps the row flags aligned
          qcol[o] = 0;
          qval[o] = 0;
        }
        continue;
      }
      double sc = gmax;
      if (per_row) {
        sc = 0.0;
        for (uint64_t k = s; k < t; k++) sc = std::max(sc, (double)m.val[k]);
      }
      uint64_t o = qptr[r];
      for (uint64_t k = s; k < t; k++) {
        int32_t q = is_signed ? q_sym(m.val[k], sc, bits) : q_uns(m.val[k], sc, bits);
        if (q != 0) {
          qcol[o] = (uint16_t)m.col[k];
          qval[o] = (int8_t)(uint8_t)(uint32_t)q;
          o++;
        }
      }
      if (o == qptr[r]) {
        // check_empty_rows (quantify_util.py:440-445) sets value 1 at a random column; the
        // column here is seeded: the row's largest |v| entry, else a hash of (seed, row).
        uint32_t c;
        int32_t v = 1;
        if (t > s) {
          uint64_t best = s;
          double ba = std::fabs((double)m.val[s]);
          for (uint64_t k = s + 1; k < t; k++) {
            double a = std::fabs((double)m.val[k]);
            if (a > ba) { ba = a; best = k; }
          }
          c = m.col[best];
          if (is_signed && m.val[best] < 0.0f) v = -1;
        } else {
          c = (uint32_t)(splitmix64(p.seed ^ (uint64_t)r) % (uint64_t)m.cols);
        }
        qcol[o] = (uint16_t)c;
        qval[o] = (int8_t)v;
        o++;
      }
    }
  });

  // ---- partitions and packets ------------------------------------------------------------------
  uint32_t parts = p.pack_parts ? p.pack_parts : 1;
  uint32_t slice = rows / parts;
  std::vector<uint64_t> part_e0(parts), part_e1(parts), part_pk(parts + 1, 0);
  for (uint32_t q = 0; q < parts; q++) {
    uint32_t r0 = q * slice, r1 = (q == parts - 1) ? rows : (q + 1) * slice;
    part_e0[q] = qptr[r0];
    part_e1[q] = qptr[r1];
    uint64_t n = part_e1[q] - part_e0[q];
    part_pk[q + 1] = part_pk[q] + (n + P - 1) / P;
  }
  const uint64_t packets = part_pk[parts];
  const uint64_t tiles = (packets + kTilePackets - 1) / kTilePackets;
  out->packets = packets;
  out->tiles = tiles;
  out->tile_bytes.assign(tiles * (uint64_t)kTileBytes, 0);
  std::vector<uint32_t> tile_flags(tiles, 0);

  const int col_base = P, val_base = 11 * P;
  const uint32_t vmask = (1u << bits) - 1u;
  parallel_for(packets, 1 << 12, [&](uint64_t gb, uint64_t ge) {
    // locate partition and row of the first element of this packet range
    uint32_t part = (uint32_t)(std::upper_bound(part_pk.begin(), part_pk.end(), gb) -
                               part_pk.begin()) - 1;
    while (part + 1 < parts && part_pk[part + 1] <= gb) part++;
    uint64_t e_first = part_e0[part] + (gb - part_pk[part]) * (uint64_t)P;
    uint32_t r = (uint32_t)(std::upper_bound(qptr.begin(), qptr.end(), e_first) -
                            qptr.begin()) - 1;
    if (r >= rows) r = rows ? rows - 1 : 0;
    Bits512 pk;
    for (uint64_t g = gb; g < ge; g++) {
      while (part + 1 < parts && part_pk[part + 1] <= g) part++;
      pk.clear();
      uint32_t nflags = 0;
      uint64_t e0 = part_e0[part] + (g - part_pk[part]) * (uint64_t)P;
      for (int j = 0; j < P; j++) {
        uint64_t e = e0 + (uint64_t)j;
        if (e >= part_e1[part]) break;  // tail slots: flag 0, col 0, val 0
        while (qptr[r + 1] <= e) r++;
        while (qptr[r] > e) r--;
        // flag_j = (row != row of the previous entry); with no empty rows that is "first
        // entry of its row", and entry 0 of the matrix compares with r_last = 0
        uint32_t flag = (e == qptr[r] && e > 0) ? 1u : 0u;
        nflags += flag;
        pk.put(j, 1, flag);
        pk.put(col_base + 10 * j, 10, qcol[e] & 0x3FFu);
        pk.put(val_base + bits * j, bits, (uint32_t)(uint8_t)qval[e] & vmask);
      }
      // scatter the 64 bytes into the tile's four 512-byte slabs
      uint64_t t = g / kTilePackets;
      uint32_t lane = (uint32_t)(g % kTilePackets);
      const uint8_t* src = reinterpret_cast<const uint8_t*>(pk.w);
      uint8_t* tb = out->tile_bytes.data() + t * (uint64_t)kTileBytes;
      for (int s = 0; s < 4; s++) std::memcpy(tb + s * 512 + lane * 16, src + s * 16, 16);
      __atomic_fetch_add(&tile_flags[t], nflags, __ATOMIC_RELAXED);
    }
  });
  out->tile_rowbase.assign(tiles + 1, 0);
  for (uint64_t t = 0; t < tiles; t++) out->tile_rowbase[t + 1] = out->tile_rowbase[t] + tile_flags[t];
  if (rows && out->tile_rowbase[tiles] != rows - 1)
    return fail(AES_ERR_INVALID, "internal: packed row count mismatch");
  if (bits == 4 && (p.flags & AES_FLAG_TENSOR)) build_tc_layout(qptr, qcol, qval, out);
  return AES_OK;
}

void untile_packets(const PackedMatrix& pm, std::vector<uint8_t>* packets) {
  packets->assign(pm.packets * 64, 0);
  for (uint64_t g = 0; g < pm.packets; g++) {
    uint64_t t = g / kTilePackets;
    uint32_t lane = (uint32_t)(g % kTilePackets);
    const uint8_t* tb = pm.tile_bytes.data() + t * (uint64_t)kTileBytes;
    for (int s = 0; s < 4; s++) std::memcpy(packets->data() + g * 64 + s * 16, tb + s * 512 + lane * 16, 16);
  }
}

}  // namespace aes

// ---------------------------------------------------------------------------------------------
// seeded synthetic matrices
// ---------------------------------------------------------------------------------------------

namespace {

struct Xoshiro256 {
  uint64_t s[4];
  explicit Xoshiro256(uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) {
      x += 0x9E3779B97F4A7C15ull;
      uint64_t z = x;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      s[i] = z ^ (z >> 31);
    }
  }
  static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
};

uint64_t row_seed(uint64_t seed, uint64_t row, uint64_t stream) {
  uint64_t z = seed * 0xD1B54A32D192ED03ull + row * 0x9E3779B97F4A7C15ull + stream * 0xA0761D6478BD642Full;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

uint32_t gen_degree(uint32_t kind, uint32_t cols, double p0, double p1, Xoshiro256& g) {
  uint32_t d = 0;
  switch (kind) {
    case AES_GEN_UNIFORM_DEG: {
      uint32_t lo = (uint32_t)p0, hi = (uint32_t)p1;
      d = lo + g.below(hi - lo + 1);
      break;
    }
    case AES_GEN_FIXED_ABSNORMAL:
    case AES_GEN_FIXED_UNIFORM:
      d = (uint32_t)p0;
      break;
    case AES_GEN_GAMMA_DEG: {
      // Gamma(shape 2, scale mean/2) = -(mean/2) * ln(U1 * U2)
      double u1 = 1.0 - g.uniform(), u2 = 1.0 - g.uniform();
      double x = -(p0 / 2.0) * std::log(u1 * u2);
      double r = std::nearbyint(x);
      if (r < 1.0) r = 1.0;
      if (r > p1) r = p1;
      d = (uint32_t)r;
      break;
    }
  }
  return std::min(d, cols);
}

}  // namespace

extern "C" uint64_t aes_gen_matrix(uint32_t kind, uint32_t rows, uint32_t cols, double p0,
                                   double p1, uint64_t seed, uint64_t* ptr, uint32_t* col,
                                   float* val) {
  if (kind > AES_GEN_FIXED_UNIFORM || cols == 0 || rows == 0) return (uint64_t)-1;
  if (kind == AES_GEN_UNIFORM_DEG && (p1 < p0 || p0 < 0)) return (uint64_t)-1;
  std::vector<uint32_t> deg(rows);
  aes::parallel_for(rows, 1 << 15, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; r++) {
      Xoshiro256 g(row_seed(seed, r, 0));
      deg[r] = gen_degree(kind, cols, p0, p1, g);
    }
  });
  uint64_t total = 0;
  for (uint32_t r = 0; r < rows; r++) total += deg[r];
  if (!ptr) return total;
  ptr[0] = 0;
  for (uint32_t r = 0; r < rows; r++) ptr[r + 1] = ptr[r] + deg[r];
  aes::parallel_for(rows, 1 << 13, [&](uint64_t b, uint64_t e) {
    std::vector<uint64_t> bm((cols + 63) / 64);
    for (uint64_t r = b; r < e; r++) {
      Xoshiro256 g(row_seed(seed, r, 1));
      uint32_t d = deg[r];
      std::fill(bm.begin(), bm.end(), 0ull);
      if (d * 2 <= cols) {
        uint32_t got = 0;
        while (got < d) {
          uint32_t c = g.below(cols);
          uint64_t bit = 1ull << (c & 63);
          if (!(bm[c >> 6] & bit)) { bm[c >> 6] |= bit; got++; }
        }
      } else {  // dense rows: choose the columns to leave out
        for (auto& w : bm) w = ~0ull;
        if (cols & 63) bm.back() = (1ull << (cols & 63)) - 1;
        uint32_t drop = cols - d, got = 0;
        while (got < drop) {
          uint32_t c = g.below(cols);
          uint64_t bit = 1ull << (c & 63);
          if (bm[c >> 6] & bit) { bm[c >> 6] &= ~bit; got++; }
        }
      }
      uint64_t o = ptr[r];
      for (size_t w = 0; w < bm.size(); w++) {
        uint64_t x = bm[w];
        while (x) {
          int bpos = __builtin_ctzll(x);
          x &= x - 1;
          col[o++] = (uint32_t)(w * 64 + bpos);
        }
      }
      for (uint64_t k = ptr[r]; k < o; k++) {
        float v;
        if (kind == AES_GEN_FIXED_ABSNORMAL) {
          double u1 = 1.0 - g.uniform(), u2 = g.uniform();
          v = (float)std::fabs(std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        } else {
          v = (float)g.uniform();
        }
        val[k] = v;
      }
    }
  });
  return total;
}
