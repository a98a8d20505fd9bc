// aes_tc_layout.h -- operand layout shared by the host packer and the tensor-core candidate pass
// of 4-bit matrices (aes_tc.cuh): 128-row (or 128-query) K-major FP8 e4m3 operands without
// swizzle, made of 8-row x 16-byte core matrices; K-adjacent core matrices lie 2048 bytes apart,
// 8-row groups 128 bytes apart.
#pragma once

#include <cstddef>
#include <cstdint>

#ifdef __CUDACC__
#define AES_HD __host__ __device__
#else
#define AES_HD
#endif

namespace aes {

constexpr uint32_t kTcRows = 128;                        // rows per tile: the MMA's M
constexpr uint32_t kTcQ = 128;                           // queries per launch: the MMA's N
constexpr uint32_t kTcChunkK = 256;                      // columns per staged chunk
constexpr uint32_t kTcChunkBytes = kTcRows * kTcChunkK;  // 32 KB of e4m3 per chunk buffer
constexpr uint32_t kTcMaxSplit = 32;                     // thresholds of <= 32 partitions in smem

AES_HD inline uint32_t tc_kpad(uint32_t cols) { return (cols + 31u) & ~31u; }
AES_HD inline uint32_t tc_nchunks(uint32_t cols) {
  return (tc_kpad(cols) + kTcChunkK - 1) / kTcChunkK;
}
// bytes of the e4m3 query operand (128 queries x kpad columns)
AES_HD inline size_t tc_qtab_bytes(uint32_t cols) { return (size_t)(tc_kpad(cols) / 16) * 2048; }
// byte offset of element (r, k) of a 128-row operand
AES_HD inline uint32_t tc_off(uint32_t r, uint32_t k) {
  return (k >> 4) * 2048u + (r >> 3) * 128u + (r & 7u) * 16u + (k & 15u);
}
// e4m3 encoding of an integer with |v| <= 16, exact: sign, 4-bit exponent biased by 7, the
// three bits after the leading one
AES_HD inline uint8_t e4m3_small(int v) {
  if (v == 0) return 0;
  const uint32_t s = v < 0 ? 0x80u : 0u;
  const uint32_t m = (uint32_t)(v < 0 ? -v : v);
  uint32_t e = 0;
  while ((m >> (e + 1)) != 0) e++;  // m in [2^e, 2^(e+1))
  const uint32_t f = ((m << 3) >> e) & 7u;
  return (uint8_t)(s | ((e + 7u) << 3) | f);
}

}  // namespace aes
