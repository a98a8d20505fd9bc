// aes_host.hpp -- host-side data preparation of the Top-K SpMV engine: FP32 CSR, quantisers,
// the seeded empty-row rule, the Ultra-CSR packer and the tile metadata the kernels need.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "acceles.h"

namespace aes {

// Ultra-CSR elements per 512-bit packet, types.hpp:161 (ULTRACSR_PACKET_SIZE with B-bit values):
// floor((512 - 1) / (B + 10 + 1)).  B=4: 34, B=6: 30, B=8: 26.
inline int packet_elems(int bits) { return 511 / (bits + 11); }

constexpr int kTilePackets = 32;                   // one packet per lane of a warp
constexpr int kTileBytes = kTilePackets * 64;      // 2 KB
constexpr uint32_t kMaxCols = 1024;                // 10-bit column field (types.hpp:58,153)

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

// Run fn(begin, end) over [0, n) on the host's cores.
void parallel_for(uint64_t n, uint64_t grain, const std::function<void(uint64_t, uint64_t)>& fn);

struct HostCSR {
  uint32_t rows = 0, cols = 0;
  std::vector<uint64_t> ptr;  // rows + 1
  std::vector<uint32_t> col;
  std::vector<float> val;     // FP32 values; empty for a pre-quantised matrix given without them
  std::vector<int8_t> qv;     // pre-quantised B-bit values (the reference's q_val), or empty
  bool prequantized = false;  // qv holds the values to pack (no quantiser)
};

// Stable (row, col) order; duplicates keep input order.  val and qval may each be null; the CSR
// carries whichever arrays were given.
int coo_to_csr(const uint32_t* row, const uint32_t* col, const float* val, uint32_t rows,
               uint32_t cols, uint64_t nnz, HostCSR* out, const int8_t* qval = nullptr);
int check_csr(const uint64_t* ptr, const uint32_t* col, uint32_t rows, uint32_t cols);

// The quantised matrix in packed form, laid out for the device.
struct PackedMatrix {
  uint32_t rows = 0, cols = 0, bits = 0, quant = 0, P = 0;
  uint64_t qnnz = 0, packets = 0, tiles = 0;
  // Tiles of 32 packets; within a tile, slab s (16-byte quarter s of every packet) is stored
  // contiguously: byte offset t*2048 + s*512 + lane*16 + (b & 15) for packet byte b,
  // s = b >> 4.  Packet bytes are exactly the reference layout (fpga_utils.hpp:438-527).
  std::vector<uint8_t> tile_bytes;
  std::vector<uint32_t> tile_rowbase;  // flags set in all packets before tile t; size tiles+1
  std::vector<float> rowscale;         // AES_QUANT_UNSIGNED_ROW only
  // Tensor-core layout (B = 4 with AES_FLAG_TENSOR and no duplicate (row, col)): the entries of
  // each 128-row tile grouped by 256-column chunk, tile-major; an entry is its byte offset in
  // the chunk operand (tc_off of the row in the tile and the column in the chunk) << 16 | its
  // e4m3 value.  tc_ptr[t * tc_nch + c] is the first entry of (tile t, chunk c).
  std::vector<uint32_t> tc_ptr, tc_ent;
  uint32_t tc_nch = 0;
};

// Quantise (quantify_util.py:8-28 or the per-row variant), drop zero results
// (matrix_to_coo), give rows left empty one entry (check_empty_rows, seeded), and pack the
// result as Ultra-CSR in pack_parts row partitions (host_spmv_ucsr.cpp:278-425).  A matrix with
// pre-quantised values (m.prequantized) is packed as given, every entry kept (Q_packet_coo packs
// the COO it is handed); a row without entries gets one entry of value 0 at column 0, so that
// the row flags still count every row and its score stays 0.
int quantize_and_pack(const HostCSR& m, const aes_params& p, PackedMatrix* out);

// Reference-order packets (partition by partition, 64 bytes each) recovered from the tiled
// layout; used by tests of the packer.
void untile_packets(const PackedMatrix& pm, std::vector<uint8_t>* packets);

}  // namespace aes
