// aes_qexact.hpp -- the query quantisers in integer arithmetic, bit-identical to their float64
// statements, so that no FP64 instruction runs on the GPU.
//
// quantify_vector (quantify_util.py:31-49) computes, in float64 on the float64 copy of each
// FP32 query value x with scale m = max |x| (or max x):
//     q = clip(round_half_even(fl64(M * fl64(x / m))), lo, M)
// fl64 is IEEE binary64 round-to-nearest-even.  Here x and m are FP32, so their significands
// have 24 bits: the quotient is formed exactly to 63 bits plus a remainder (two 64-bit
// divisions), rounded to 53 bits as binary64 division would; the product by M (at most 8 bits)
// is exact in 64 bits and is rounded to 53 bits as binary64 multiplication would; the last
// step rounds to an integer, ties to even.  Binary64 has neither overflow nor subnormals here
// (|x / m| <= 1 and >= 2^-277).
//
// quantize_vec (quantize_utils.hpp:8-18) truncates x * 2^30 toward zero and keeps the low 32
// bits (two's-complement wrap); x * 2^30 is exact, so the integer part is a shift of x's
// significand.
#pragma once

#include <stdint.h>

#include <cstring>

#ifdef __CUDACC__
#define AES_QX_FN __host__ __device__ __forceinline__
#else
#define AES_QX_FN inline
#endif

namespace aes {
namespace qx {

AES_QX_FN uint32_t fbits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}

AES_QX_FN int bitlen64(uint64_t v) {
#ifdef __CUDA_ARCH__
  return v ? 64 - __clzll((long long)v) : 0;
#else
  return v ? 64 - __builtin_clzll(v) : 0;
#endif
}

// |f| = sig * 2^exp with sig in [2^23, 2^24) (subnormals normalised); f must be finite, nonzero
AES_QX_FN void unpack(float f, uint64_t* sig, int* exp) {
  const uint32_t u = fbits(f);
  const int e = (int)((u >> 23) & 0xFFu);
  uint64_t m = u & 0x7FFFFFu;
  int x;
  if (e == 0) {
    x = -149;
    while (m < (1ull << 23)) {
      m <<= 1;
      x--;
    }
  } else {
    m |= 1ull << 23;
    x = e - 150;
  }
  *sig = m;
  *exp = x;
}

// v * 2^exp with v < 2^64 rounded to 53 significant bits, ties to even (extra = a nonzero
// remainder below v's last bit); returns the 53-bit significand, adjusts *exp
AES_QX_FN uint64_t round53(uint64_t v, bool extra, int* exp) {
  const int L = bitlen64(v);
  if (L <= 53) return v;  // exact (extra is then zero in every use below)
  const int s = L - 53;
  uint64_t m = v >> s;
  const uint64_t rem = v & ((1ull << s) - 1ull), half = 1ull << (s - 1);
  if (rem > half || (rem == half && (extra || (m & 1ull)))) m++;
  *exp += s;
  if (m == (1ull << 53)) {
    m >>= 1;
    *exp += 1;
  }
  return m;
}

// round_half_even(fl64(M * fl64(x / m))) for FP32 x, m > 0 and integer 1 <= M <= 255
AES_QX_FN int32_t round_scaled(float x, float m, int32_t M) {
  if (x == 0.0f) return 0;
  const bool neg = x < 0.0f;
  uint64_t X, Y;
  int ex, ey;
  unpack(x, &X, &ex);
  unpack(m, &Y, &ey);
  // floor(X * 2^62 / Y) in two steps, and whether a remainder is left
  const uint64_t n1 = X << 39;
  const uint64_t q1 = n1 / Y, r1 = n1 % Y;
  const uint64_t n2 = r1 << 23;
  const uint64_t q2 = n2 / Y, r2 = n2 % Y;
  const uint64_t Q = (q1 << 23) | q2;  // in (2^61, 2^63)
  int e = ex - ey - 62;
  const uint64_t d = round53(Q, r2 != 0, &e);  // fl64(x / m) = d * 2^e
  const uint64_t P = (uint64_t)M * d;          // exact: < 2^61
  const uint64_t p = round53(P, false, &e);     // fl64(M * ...) = p * 2^e
  uint64_t q;
  if (e >= 0) {
    q = p << e;
  } else {
    const int s = -e;
    if (s >= 64) {
      q = 0;  // below 2^-11
    } else {
      q = p >> s;
      const uint64_t rem = p & ((1ull << s) - 1ull), half = 1ull << (s - 1);
      if (rem > half || (rem == half && (q & 1ull))) q++;
    }
  }
  const int32_t r = (int32_t)q;
  return neg ? -r : r;
}

// low 32 bits of trunc(x * 2^30) (two's complement), for finite x
AES_QX_FN int32_t trunc_scaled30(float x) {
  if (x == 0.0f) return 0;
  const bool neg = x < 0.0f;
  uint64_t X;
  int ex;
  unpack(x, &X, &ex);
  const int s = ex + 30;  // |x| * 2^30 = X * 2^s
  uint32_t t;
  if (s >= 32) t = 0u;                       // a multiple of 2^32
  else if (s >= 0) t = (uint32_t)(X << s);   // low 32 bits
  else if (s > -64) t = (uint32_t)(X >> -s);
  else t = 0u;
  return (int32_t)(neg ? 0u - t : t);
}

}  // namespace qx
}  // namespace aes
