/* Accuracy of the contract's transcendental functions (rfmm_math.h) against
 * double-precision libm, in units in the last place of the binary32 result,
 * over seeded random arguments in the ranges the solver's passes use.
 * Prints one line: the maximum error of each function. */
#include <stdio.h>
#include <stdlib.h>

#include "rfmm_math.h"

static double ulp_of(double v) {
  double a = fabs(v);
  if (a < 1e-30) a = 1e-30;
  int e;
  frexp(a, &e);
  return ldexp(1.0, e - 24);
}

static unsigned long long state = 88172645463325252ull;
static double uniform01(void) { /* xorshift64 */
  state ^= state << 13;
  state ^= state >> 7;
  state ^= state << 17;
  return (double)(state >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char **argv) {
  const long samples = argc > 1 ? atol(argv[1]) : 2000000;
  double ms = 0, mc = 0, me = 0, ml = 0, mp = 0, ma = 0;
  for (long i = 0; i < samples; i++) {
    const float x = (float)((uniform01() - 0.5) * 80.0); /* seed angles reach ~40 */
    const double s = sin((double)x), c = cos((double)x);
    if (fabs(s) > 1e-3) { const double e = fabs(rf_sinf(x) - s) / ulp_of(s); if (e > ms) ms = e; }
    if (fabs(c) > 1e-3) { const double e = fabs(rf_cosf(x) - c) / ulp_of(c); if (e > mc) mc = e; }
    const float xe = (float)(-uniform01() * 80.0); /* control field / tone map: e^-t */
    { const double r = exp((double)xe); const double e = fabs(rf_expf(xe) - r) / ulp_of(r); if (e > me) me = e; }
    const float xp = (float)uniform01(), yp = (float)(0.2 + 3.0 * uniform01());
    if (xp > 1e-6f) {
      const double r = pow((double)xp, (double)yp), l = log((double)xp);
      const double e = fabs(rf_powf(xp, yp) - r) / ulp_of(r);
      if (e > mp) mp = e;
      if (fabs(l) > 1e-3) { const double el = fabs(rf_logf(xp) - l) / ulp_of(l); if (el > ml) ml = el; }
    }
    const float ay = (float)((uniform01() - 0.5) * 4.0), ax = (float)((uniform01() - 0.5) * 4.0);
    const double r = atan2((double)ay, (double)ax);
    if (fabs(r) > 1e-3) { const double e = fabs(rf_atan2f(ay, ax) - r) / ulp_of(r); if (e > ma) ma = e; }
  }
  printf("sin %.2f cos %.2f exp %.2f log %.2f pow %.2f atan2 %.2f\n", ms, mc, me, ml, mp, ma);
  return 0;
}
