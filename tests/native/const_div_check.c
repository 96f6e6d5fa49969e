/* Exhaustive check of the kernels' division by a constant divisor.
 *
 * The body kernels replace x / c (c = 1.6f, the world half extent, and
 * c = 0.70f - 0.30f, the excitation smoothstep width) by the quotient
 * estimate q0 = RN(x * z), z = RN(1 / c), corrected once with the exact
 * remainder: r = fma(-q0, c, x), q = fma(r, z, q0) (Markstein's correction
 * step; Brisebarre, Muller & Raina 2004 for constant divisors).  Inputs with
 * |x| < 2^-100, where the remainder is not representable, keep the division;
 * non-finite estimates are returned as they are.  This program compares the
 * result with IEEE division for every non-negative binary32 input (the
 * method is symmetric in the sign) and prints the mismatch count per
 * divisor; the test requires zero.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

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

static float div_by_const(float x, float c, float z) {
  if (fabsf(x) < 0x1p-100f) return x / c;
  const float q0 = x * z;
  if (!(fabsf(q0) < INFINITY)) return q0;
  const float r = fmaf(-q0, c, x);
  return fmaf(r, z, q0);
}

int main(void) {
  volatile float hi = 0.70f, lo = 0.30f;
  const float divisors[2] = {1.60f, hi - lo};
  int status = 0;
  for (int k = 0; k < 2; k++) {
    const float c = divisors[k];
    const float z = 1.0f / c;
    long long bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
    for (long long i = 0; i < (1ll << 31); i++) {
      const float x = from_bits((uint32_t)i);
      const float want = x / c, got = div_by_const(x, c, z);
      if (to_bits(got) != to_bits(want) && !(isnan(got) && isnan(want))) bad++;
    }
    printf("divisor 0x%08x reciprocal 0x%08x mismatches %lld\n", to_bits(c), to_bits(z), bad);
    if (bad) status = 1;
  }
  return status;
}
