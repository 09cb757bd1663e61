/* Checks, on the CPU, the division used by the GPU voxel walks: the quotient
 * x / d formed from the correctly rounded reciprocal r = RN(1/d) as
 *   q = RN(x * r),  e = x - d * q (one FMA),  result = RN(q + e * r)
 * (Markstein's theorem), against IEEE single-precision division, over the
 * walks' domain: 2^-24 <= |x| <= 2 (distance to the next grid plane) and
 * 2^-60 <= |d| <= 2^60 (direction components).  Built with FMA contraction
 * off so that every operation is rounded as written.
 * Returns the number of mismatching pairs; prints the first few. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static uint64_t state = 0x9E3779B97F4A7C15ull;
static uint64_t next(void) {
  state ^= state << 13;
  state ^= state >> 7;
  state ^= state << 17;
  return state;
}
static float from_bits(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static uint32_t to_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}
static float div_by_recip(float x, float d) {
  const float r = 1.0f / d;
  const float q = x * r;
  const float e = fmaf(-q, d, x);
  return fmaf(e, r, q);
}
static long long check(float x, float d, long long bad) {
  const float a = x / d, b = div_by_recip(x, d);
  if (to_bits(a) != to_bits(b)) {
    if (bad < 5) printf("mismatch x=%a d=%a: %a vs %a\n", x, d, a, b);
    return 1;
  }
  return 0;
}

long long markstein_check(long long random_pairs, long long sweep) {
  long long bad = 0;
  for (long long i = 0; i < random_pairs; ++i) {
    const uint64_t r = next();
    /* d: exponent in [-60, 60], any mantissa, either sign */
    const uint32_t de = (uint32_t)(127 - 60 + (r >> 24) % 121);
    const float d = from_bits((uint32_t)(r & 0x7fffff) | (de << 23) | ((uint32_t)(r >> 63) << 31));
    /* x: exponent in [-24, 0], any mantissa, either sign; plus x in [1, 2] */
    const uint64_t s = next();
    const uint32_t xe = (uint32_t)(127 - 24 + (s >> 24) % 25);
    const float x = from_bits((uint32_t)(s & 0x7fffff) | (xe << 23) | ((uint32_t)(s >> 63) << 31));
    bad += check(x, d, bad);
    bad += check(from_bits(0x3f800000u | (uint32_t)(s >> 40 & 0x7fffff)), d, bad);
  }
  /* mantissa sweeps: x over [1,2) for fixed unit-range d, d over [1,2) for fixed x */
  static const float ds[] = {0.3f, -0.70710677f, 1e-7f, 0.99999994f, -3.3e-5f, 0.57735026f};
  static const float xs[] = {1.0f, 0.999f, -0.123456f, 3.0e-7f, 1.9999999f, 5.9604645e-8f};
  for (int j = 0; j < 6; ++j)
    for (long long m = 0; m < sweep; ++m) {
      const uint32_t mm = (uint32_t)(m * (0x800000 / sweep));
      bad += check(from_bits(0x3f800000u | mm), ds[j], bad);
      bad += check(xs[j], from_bits(0x3f800000u | mm), bad);
    }
  return bad;
}
