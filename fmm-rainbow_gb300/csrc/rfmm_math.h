/*
 * rfmm_math.h -- the transcendental functions of the solver's floating-point
 * contract (binary32), compiled identically as CUDA device code and as C.
 *
 * The reference's WGSL sin/cos/exp/pow/atan2 are implementation-defined (the
 * WebGPU spec bounds their error, nothing more).  The seed (wgsl:232-374), the
 * control field (wgsl:659-689) and the display passes (wgsl:780-1009) use these
 * definitions instead, so the GPU and the CPU oracle agree bit for bit.  Every
 * function is a fixed sequence of IEEE binary32 operations with explicit fused
 * multiply-adds (no contraction is left to the compiler), written from the
 * functions' series:
 *   sin, cos  Cody-Waite reduction by pi/2 (three-part constant), Taylor
 *             polynomials to degree 9 / 10 on [-pi/4, pi/4]
 *   exp       reduction by ln 2 (two-part constant), Taylor to degree 7 on
 *             [-ln2/2, ln2/2], exponent scaling
 *   log2      mantissa in [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1)),
 *             odd series to degree 11
 *   pow       exp(y ln x) for x >= 0
 *   atan2     octant reduction, atan(t) = pi/6 + atan((t sqrt3 - 1)/(t + sqrt3))
 *             above tan(pi/12), odd Taylor series to degree 15
 * Accuracy (checked against double-precision libm in the tests): a few units
 * in the last place over the arguments these passes use.
 */
#ifndef RFMM_MATH_H
#define RFMM_MATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

/* fmaf is the IEEE fused multiply-add on both sides (libm on the host, the
 * hardware FFMA on the device); rintf rounds to nearest even on both. */
#ifdef __CUDACC__
#define RF_FN __host__ __device__ __forceinline__
#else
#define RF_FN static inline
#endif
#define RF_FMA(a, b, c) fmaf((a), (b), (c))
#define RF_RINT(x) rintf(x)

RF_FN float rf_bits_to_float(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

RF_FN uint32_t rf_float_to_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

/* x * 2^n for an integer n in [-252, 254], exact unless the result is subnormal. */
RF_FN float rf_scale2(float x, int n) {
  if (n > 127) {
    x = x * rf_bits_to_float(0x7F000000u); /* 2^127 */
    n -= 127;
    if (n > 127) n = 127;
  } else if (n < -126) {
    x = x * rf_bits_to_float(0x00800000u); /* 2^-126 */
    n += 126;
    if (n < -126) n = -126;
  }
  return x * rf_bits_to_float((uint32_t)(n + 127) << 23);
}

/* sin and cos of x, |x| < 2^15. */
RF_FN void rf_sincosf(float x, float *s, float *c) {
  /* pi/2 = C1 + C2 + C3, C1 and C2 with 12 significant bits, so k * C1 and
   * k * C2 are exact for |k| < 2^11 */
  const float k = RF_RINT(x * 0x1.45f306p-1f);  /* x * RN(2/pi) */
  float r = RF_FMA(-k, 0x1.922p+0f, x);         /* C1 = 1.57080078125 */
  r = RF_FMA(-k, -0x1.2aep-18f, r);             /* C2 = -4.45358455e-6 */
  r = RF_FMA(-k, -0x1.de973ep-31f, r);          /* C3 = -8.705516e-10 */
  const float r2 = r * r;
  /* sin r = r + r^3 (-1/3! + r^2 (1/5! + r^2 (-1/7! + r^2 / 9!))) */
  float ps = RF_FMA(r2, 2.75573192e-06f, -1.98412698e-04f);
  ps = RF_FMA(r2, ps, 8.33333333e-03f);
  ps = RF_FMA(r2, ps, -1.66666667e-01f);
  const float sn = RF_FMA(r * r2, ps, r);
  /* cos r = 1 - r^2/2 + r^4 (1/4! + r^2 (-1/6! + r^2 (1/8! - r^2 / 10!))) */
  float pc = RF_FMA(r2, -2.75573192e-07f, 2.48015873e-05f);
  pc = RF_FMA(r2, pc, -1.38888889e-03f);
  pc = RF_FMA(r2, pc, 4.16666667e-02f);
  const float cs = RF_FMA(r2 * r2, pc, RF_FMA(r2, -0.5f, 1.0f));
  const int q = ((int)k) & 3;
  if (q == 0) {
    *s = sn;
    *c = cs;
  } else if (q == 1) {
    *s = cs;
    *c = -sn;
  } else if (q == 2) {
    *s = -sn;
    *c = -cs;
  } else {
    *s = -cs;
    *c = sn;
  }
}

RF_FN float rf_sinf(float x) {
  float s, c;
  rf_sincosf(x, &s, &c);
  return s;
}

RF_FN float rf_cosf(float x) {
  float s, c;
  rf_sincosf(x, &s, &c);
  return c;
}

/* e^x. */
RF_FN float rf_expf(float x) {
  if (!(x == x)) return x;
  if (x > 88.8f) return rf_bits_to_float(0x7F800000u);
  if (x < -104.0f) return 0.0f;
  /* ln 2 = L1 + L2, L1 with 16 significant bits (k * L1 exact) */
  const float k = RF_RINT(x * 0x1.715476p+0f);  /* x * RN(1/ln 2) */
  float r = RF_FMA(-k, 0x1.62e4p-1f, x);        /* L1 = 0.693145752 */
  r = RF_FMA(-k, 0x1.7f7d1cp-20f, r);           /* L2 = 1.42860677e-6 */
  /* e^r = 1 + r + r^2/2! + ... + r^7/7! */
  float p = RF_FMA(r, 1.98412698e-04f, 1.38888889e-03f);
  p = RF_FMA(r, p, 8.33333333e-03f);
  p = RF_FMA(r, p, 4.16666667e-02f);
  p = RF_FMA(r, p, 1.66666667e-01f);
  p = RF_FMA(r, p, 0.5f);
  p = RF_FMA(r, p, 1.0f);
  p = RF_FMA(r, p, 1.0f);
  return rf_scale2(p, (int)k);
}

/* ln x for finite x > 0 (subnormals included). */
RF_FN float rf_logf(float x) {
  uint32_t u = rf_float_to_bits(x);
  int e = 0;
  if (u < 0x00800000u) { /* subnormal: normalise */
    x = x * 16777216.0f;
    u = rf_float_to_bits(x);
    e = -24;
  }
  e += (int)(u >> 23) - 127;
  float m = rf_bits_to_float((u & 0x007FFFFFu) | 0x3F800000u); /* [1, 2) */
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  /* ln m = 2 (s + s^3/3 + s^5/5 + s^7/7 + s^9/9 + s^11/11) */
  float p = RF_FMA(s2, 9.09090909e-02f, 1.11111111e-01f);
  p = RF_FMA(s2, p, 1.42857143e-01f);
  p = RF_FMA(s2, p, 2.0e-01f);
  p = RF_FMA(s2, p, 3.33333333e-01f);
  const float lnm = 2.0f * RF_FMA(s * s2, p, s);
  const float fe = (float)e;
  /* e ln 2 + ln m with ln 2 in two parts */
  return RF_FMA(fe, 0x1.62e4p-1f, RF_FMA(fe, 0x1.7f7d1cp-20f, lnm));
}

/* x^y for x >= 0 (x = 0: 0 for y > 0, 1 for y = 0). */
RF_FN float rf_powf(float x, float y) {
  if (y == 0.0f || x == 1.0f) return 1.0f;
  if (x == 0.0f) return y > 0.0f ? 0.0f : rf_bits_to_float(0x7F800000u);
  return rf_expf(y * rf_logf(x));
}

/* atan2(y, x) in (-pi, pi]; atan2(0, 0) = 0. */
RF_FN float rf_atan2f(float y, float x) {
  const float ax = x < 0.0f ? -x : x, ay = y < 0.0f ? -y : y;
  const float hi = ax > ay ? ax : ay, lo = ax > ay ? ay : ax;
  if (hi == 0.0f) return 0.0f;
  float t = lo / hi; /* [0, 1] */
  float base = 0.0f;
  if (t > 0.267949192f) { /* tan(pi/12) */
    t = (t * 1.73205081f - 1.0f) / (t + 1.73205081f);
    base = 0.523598776f; /* pi/6 */
  }
  const float t2 = t * t;
  /* atan t = t - t^3/3 + t^5/5 - ... - t^15/15 */
  float p = RF_FMA(t2, -6.66666667e-02f, 7.69230769e-02f);
  p = RF_FMA(t2, p, -9.09090909e-02f);
  p = RF_FMA(t2, p, 1.11111111e-01f);
  p = RF_FMA(t2, p, -1.42857143e-01f);
  p = RF_FMA(t2, p, 2.0e-01f);
  p = RF_FMA(t2, p, -3.33333333e-01f);
  float a = base + RF_FMA(t * t2, p, t);
  if (ay > ax) a = 1.57079633f - a;
  if (x < 0.0f) a = 3.14159265f - a;
  return y < 0.0f ? -a : a;
}

#endif /* RFMM_MATH_H */
