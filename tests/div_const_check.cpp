// Host check of pda::div_const (Markstein's correctly rounded division by a
// constant) against IEEE division: random doubles over the exponent range the
// WENO5 gradients see (and far beyond), both signs, zeros.  Prints the number
// of mismatches; built and run by tests/test_div_const.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "numerics.cuh"

static bool same(double a, double b) {
  uint64_t x, y;
  std::memcpy(&x, &a, 8);
  std::memcpy(&y, &b, 8);
  return x == y || (a == 0. && b == 0.);
}

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> mant(1.0, 2.0);
  std::uniform_int_distribution<int> ex(-900, 900);
  long bad = 0, n = 0;
  const double ds[2] = {3., 6.};
  for (long i = 0; i < 4000000; ++i) {
    double x = std::ldexp(mant(rng), ex(rng));
    if (i & 1) x = -x;
    for (double d : ds) {
      const double got = pda::div_const(x, d, 1. / d);
      if (!same(got, x / d)) ++bad;
      ++n;
    }
  }
  // integers and small multiples (exact quotients and ties of the neighbourhood)
  for (long k = -200000; k <= 200000; ++k) {
    const double x = (double)k * 0.125;
    for (double d : ds) {
      if (!same(pda::div_const(x, d, 1. / d), x / d)) ++bad;
      ++n;
    }
  }
  std::printf("%ld %ld\n", bad, n);
  return 0;
}
