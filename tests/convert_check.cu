// Host check of the integer FP32 <-> FP64 conversions of the mixed sweep
// (fest_convert.cuh) against the compiler's conversions: random bit
// patterns, doubles over the FP32 exponent range, exact rounding ties and
// their neighbours; prints the mismatch counts.
#include <math.h>
#include <stdio.h>

#include "fest_convert.cuh"

static unsigned long long s = 0x9e3779b97f4a7c15ull;
static unsigned long long next() {  // splitmix64
  unsigned long long z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

int main() {
  long long bad_f2d = 0, bad_d2f = 0, n = 1 << 22;
  for (long long t = 0; t < n; ++t) {
    const unsigned long long r = next();
    const float f = fest::f32_from((unsigned)r);
    const unsigned fe = ((unsigned)r >> 23) & 0xffu;
    if (fe != 0u && f == f) {  // normal numbers and infinities
      const double a = fest::f2d(f), b = (double)f;
      if (memcmp(&a, &b, sizeof a) != 0) ++bad_f2d;
    }
    const unsigned long long r2 = next();
    const int ex = (int)(r2 % 300) - 150;
    double d = ldexp(1.0 + (double)(r2 >> 12) * (1.0 / 4503599627370496.0), ex) * ((r2 & 1) ? -1.0 : 1.0);
    if (r2 % 7 == 0 && f == f && !isinf(f)) d = (double)f + ldexp((double)((r2 >> 20) & 0xffff) - 32768.0, -60) * fabs((double)f);
    const float c = fest::d2f(d), e = (float)d;
    const bool normal_out = fabs((double)e) >= 1.1754943508222875e-38 || e == 0.0f;
    if (normal_out && memcmp(&c, &e, sizeof c) != 0) ++bad_d2f;
    // exact ties between two adjacent floats, and their neighbours
    if (fe != 0u && fe < 0xfeu) {
      const float g = nextafterf(f, INFINITY);
      const double mid = 0.5 * ((double)f + (double)g);  // exact in FP64
      const double ds[3] = {mid, nextafter(mid, INFINITY), nextafter(mid, -INFINITY)};
      for (double x : ds) {
        const float c2 = fest::d2f(x), e2 = (float)x;
        if (memcmp(&c2, &e2, sizeof c2) != 0) ++bad_d2f;
      }
    }
  }
  printf("%lld %lld %lld\n", n, bad_f2d, bad_d2f);
  return 0;
}
