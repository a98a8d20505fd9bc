// Checks the integer query quantisers of aes_qexact.hpp against float64 arithmetic on the CPU:
// round_half_even(M * (x / m)) in binary64, and the low 32 bits of trunc(x * 2^30).
// Prints the number of mismatches (0 expected) and exits non-zero on any.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "aes_qexact.hpp"

static int32_t ref_round(float x, float m, int32_t M) {
  const double d = (double)x / (double)m;
  const double y = (double)M * d;
  return (int32_t)std::nearbyint(y);
}

static int32_t ref_trunc(float x) {
  const double v = std::ldexp((double)x, 30);
  if (std::fabs(v) >= 9.2e18) return 0;  // outside int64: the low 32 bits are zero
  const int64_t t = (int64_t)std::trunc(v);
  return (int32_t)(uint32_t)(uint64_t)t;
}

static float from_bits(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
  std::mt19937_64 g(12345);
  std::uniform_real_distribution<float> U(0.0f, 1.0f);
  const int32_t Ms[] = {1, 3, 7, 15, 31, 63, 127, 255};
  long bad = 0, ties = 0, checked = 0;
  for (long i = 0; i < n; i++) {
    const int32_t M = Ms[g() % 8];
    float m, x;
    switch (i % 5) {
      case 0: {  // random value in [-m, m]
        m = std::ldexp(0.5f + U(g), (int)(g() % 80) - 40);
        x = (U(g) * 2.0f - 1.0f) * m;
        break;
      }
      case 1: {  // near a tie: x ~ m * (k + 1/2) / M, nudged by a few ulps
        m = std::ldexp(0.5f + U(g), (int)(g() % 60) - 30);
        const int k = (int)(g() % (uint64_t)M);
        x = (float)((double)m * (k + 0.5) / M);
        uint32_t u;
        std::memcpy(&u, &x, 4);
        u += (uint32_t)((int)(g() % 7) - 3);
        x = from_bits(u);
        if (std::fabs(x) > m) x = m;
        break;
      }
      case 2: {  // exact multiples m * j / M and m itself
        m = std::ldexp(0.5f + U(g), (int)(g() % 60) - 30);
        const int j = (int)(g() % (uint64_t)(M + 1));
        x = (float)((double)m * j / M);
        if (g() & 1) x = -x;
        break;
      }
      case 3: {  // subnormal and tiny values
        m = std::ldexp(0.5f + U(g), -(int)(g() % 30) - 100);
        x = from_bits((uint32_t)(g() % 0x00800000u)) * ((g() & 1) ? 1.0f : -1.0f);
        if (std::fabs(x) > m) x = m;
        break;
      }
      default: {  // arbitrary bit patterns with |x| <= m
        m = from_bits(0x00800000u + (uint32_t)(g() % 0x7E000000u));
        x = from_bits((uint32_t)(g() % 0x7F000000u));
        if (x > m) std::swap(x, m);
        if (g() & 1) x = -x;
        break;
      }
    }
    if (!(m > 0.0f) || !std::isfinite(m) || !std::isfinite(x)) continue;
    const int32_t a = aes::qx::round_scaled(x, m, M), b = ref_round(x, m, M);
    const double y = (double)M * ((double)x / (double)m);
    if (y - std::floor(y) == 0.5) ties++;
    checked++;
    if (a != b) {
      if (bad < 10) std::printf("round x=%a m=%a M=%d: got %d want %d\n", x, m, M, a, b);
      bad++;
    }
    const float t = from_bits((uint32_t)g());
    if (std::isfinite(t)) {
      const int32_t c = aes::qx::trunc_scaled30(t), d = ref_trunc(t);
      if (c != d) {
        if (bad < 10) std::printf("trunc x=%a: got %d want %d\n", t, c, d);
        bad++;
      }
    }
  }
  std::printf("checked %ld ties %ld mismatches %ld\n", checked, ties, bad);
  return bad ? 1 : 0;
}
