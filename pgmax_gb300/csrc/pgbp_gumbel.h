// The Gumbel(0, 1) noise stream of perturb-and-MAP runs (pgbp_gumbel, pgbp_run_perturbed).
//
// Draw number c (c = b * n + i for instance b, variable state i of an [batch, n] array) of seed s:
//   state0 = mix64(s),  r = mix64(state0 + (c + 1) * 0x9E3779B97F4A7C15)   (64-bit wraparound)
//   u = (2 * (r >> 41) + 1) * 2^-24             a float in (0, 1), exact: 2^23 equally spaced values
//   g = -ln(-ln(u))
// mix64 is the SplitMix64 output function (G. Steele, D. Lea, C. Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014); r is output c + 1 of SplitMix64 started at
// state0, so any draw is computed on its own, in any order, by any thread. ln is the function below,
// written with single-precision additions, multiplications and one division, each correctly
// rounded and none fused, so the stream is the same bit for bit on the GPU and on any host that
// evaluates float32 expressions as written (C without FP contraction, NumPy float32).
//
// ln(x), x > 0 normal: x = m 2^e with m in [sqrt(2) / 2, sqrt(2)] (exact, from the bits);
// ln(m) = 2 atanh(s), s = (m - 1) / (m + 1), |s| <= 0.172, by the series
// atanh(s) = s (1 + z / 3 + z^2 / 5 + z^3 / 7 + z^4 / 9), z = s^2 (Abramowitz and Stegun 4.1.27);
// the first omitted term is below 5e-10 of the sum. ln(x) = e ln(2) + ln(m), within a few units in
// the last place of float32 over the range used here ([6e-8, 17]).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PGBP_HD __host__ __device__ __forceinline__
#else
#define PGBP_HD inline
#endif

namespace pgbp {

PGBP_HD uint64_t gumbel_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

PGBP_HD float gumbel_bits_to_float(uint32_t u) {
  union {
    uint32_t u;
    float f;
  } v;
  v.u = u;
  return v.f;
}

PGBP_HD uint32_t gumbel_float_to_bits(float f) {
  union {
    float f;
    uint32_t u;
  } v;
  v.f = f;
  return v.u;
}

// Natural logarithm of a positive normal float (see above).
PGBP_HD float gumbel_ln(float x) {
  const uint32_t bits = gumbel_float_to_bits(x);
  int e = (int)((bits >> 23) & 0xffu) - 127;
  float m = gumbel_bits_to_float((bits & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 0x1.6a09e6p+0f) {  // sqrt(2) rounded to float
    m = m * 0.5f;
    e += 1;
  }
  const float num = m - 1.0f;
  const float den = m + 1.0f;
  const float s = num / den;
  const float z = s * s;
  float p = 0x1.c71c72p-4f;       // 1/9
  p = p * z + 0x1.24924ap-3f;     // 1/7
  p = p * z + 0x1.99999ap-3f;     // 1/5
  p = p * z + 0x1.555556p-2f;     // 1/3
  p = p * z + 1.0f;
  const float ln_m = (s * p) * 2.0f;
  return (float)e * 0x1.62e430p-1f + ln_m;  // e ln(2) + ln(m)
}

// Key of a seed: the state SplitMix64 starts from.
PGBP_HD uint64_t gumbel_key(uint64_t seed) { return gumbel_mix64(seed); }

// Draw number c of the stream with key `key`.
PGBP_HD float gumbel_draw(uint64_t key, uint64_t c) {
  const uint64_t r = gumbel_mix64(key + (c + 1ull) * 0x9E3779B97F4A7C15ull);
  const uint32_t k = (uint32_t)(r >> 41);                        // 23 bits
  const float u = (float)(2u * k + 1u) * 0x1.0p-24f;             // exact
  const float w = -gumbel_ln(u);                                  // in [6e-8, 16.7]
  return -gumbel_ln(w);
}

}  // namespace pgbp
