// rcp_f64 (csrc/swc_fpconv.h): Newton-Raphson reciprocal against the IEEE division.
// The two steps are driven from seeds 1/x (1 + d) with |d| up to 2^-20 (wider than the
// device's approximate FP32 reciprocal gives) and from the host's own seed, on random
// magnitudes across the fast range and both signs; the result must lie within one ulp
// of 1.0 / x. Built and run by test_fpconv.py.
#include "swc_fpconv.h"
#include <cmath>
#include <cstdio>
#include <random>
#ifndef ITERS
#define ITERS 1000000
#endif
int main() {
  std::mt19937_64 rng(7);
  long bad = 0, n = 0;
  double worst = 0.0;
  auto ulp_err = [](double a, double ref) {
    const double u = std::nextafter(std::fabs(ref), INFINITY) - std::fabs(ref);
    return std::fabs(a - ref) / u;
  };
  auto chk = [&](double got, double x) {
    const double ref = 1.0 / x, err = ulp_err(got, ref);
    if (err > worst) worst = err;
    if (!(err <= 1.0)) {
      if (bad < 5) printf("x %a: %a vs %a (%.3g ulp)\n", x, got, ref, err);
      ++bad;
    }
    ++n;
  };
  std::uniform_real_distribution<double> mant(1.0, 2.0), dev(-1.0, 1.0);
  for (int i = 0; i < ITERS; ++i) {
    double x = std::ldexp(mant(rng), (int)(rng() % 240) - 120);
    if (rng() & 1) x = -x;
    chk(swc::rcp_f64(x), x);
    const double d = std::ldexp(dev(rng), -20);
    chk(swc::rcp_f64_from_seed(x, (1.0 / x) * (1.0 + d)), x);
  }
  const double ed[] = {1.0, -1.0, 3.0, 1e-30, 1e30, 0.001, 48.0, 1.5, 0.1};
  for (double x : ed) chk(swc::rcp_f64(x), x);
  // outside the fast range: the IEEE division itself
  const double far[] = {0.0, 1e-300, 1e300, INFINITY};
  for (double x : far) {
    const double a = swc::rcp_f64(x), b = 1.0 / x;
    if (!(a == b)) ++bad;
    ++n;
  }
  printf("checked %ld, worst %.3f ulp, rcp mismatches %ld\n", n, worst, bad);
  return bad != 0;
}
