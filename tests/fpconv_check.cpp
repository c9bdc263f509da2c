// Bit-exactness of the integer FP32 <-> FP64 conversions against the C casts, on random
// bit patterns, random normal magnitudes and the edge values (zeros, FLT_MIN/MAX,
// overflow to infinity, subnormal results, ties). Built and run by test_fpconv.py.
#include "swc_fpconv.h"
#include <cstdio>
#include <random>
#include <cmath>
#include <cfloat>
#ifndef ITERS
#define ITERS 2000000
#endif
int main() {
  std::mt19937_64 rng(1);
  long bad = 0, n = 0;
  auto chk_n = [&](double x) { float a = swc::narrow_f64(x), b = (float)x; uint32_t ua, ub; memcpy(&ua,&a,4); memcpy(&ub,&b,4); if (ua != ub && !(std::isnan(a) && std::isnan(b))) { if (bad < 5) printf("narrow %a: %a vs %a\n", x, a, b); ++bad; } ++n; };
  auto chk_w = [&](float x) { double a = swc::widen_f32(x), b = (double)x; uint64_t ua, ub; memcpy(&ua,&a,8); memcpy(&ub,&b,8); if (ua != ub && !(std::isnan(a) && std::isnan(b))) { if (bad < 5) printf("widen %a\n", x); ++bad; } ++n; };
  for (int i = 0; i < ITERS; ++i) { uint64_t u = rng(); double x; memcpy(&x, &u, 8); chk_n(x); uint32_t v = (uint32_t)u; float y; memcpy(&y, &v, 4); chk_w(y); }
  for (int i = 0; i < ITERS; ++i) { double x = std::ldexp((double)(rng() >> 11) / 9007199254740992.0 + 0.5, (int)(rng() % 300) - 150); if (rng() & 1) x = -x; chk_n(x); chk_w((float)x); }
  const double ed[] = {0.0, -0.0, 1.0, -1.0, FLT_MAX, -FLT_MAX, (double)FLT_MAX * (1 + 1e-9), 3.4028235677973366e38, 3.4028235677973362e38, FLT_MIN, FLT_MIN * 0.5, 1e-40, INFINITY, -INFINITY, NAN, DBL_MAX, DBL_MIN, 1.0 + 1.0/16777216.0, 1.0 + 3.0/16777216.0, 1.0 + 1.0/16777216.0 + 1e-30};
  for (double x : ed) { chk_n(x); chk_w((float)x); }
  printf("checked %ld, mismatches %ld\n", n, bad);
  return bad != 0;
}
