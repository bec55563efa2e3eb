// Host build of the integer-pipe comparisons of hiten_gb300/csrc/hg_crmath.cuh
// compared with the IEEE comparisons on special values (signed zeros,
// subnormals, the step control's constants and their neighbours, infinities,
// NaNs of both signs and several payloads) and on random bit patterns.
// Prints the number of checks and of mismatches.
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "hg_crmath.cuh"

static double from_bits(uint64_t b) {
  double x;
  memcpy(&x, &b, 8);
  return x;
}

static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t rnd() {  // xorshift64*
  s ^= s >> 12;
  s ^= s << 25;
  s ^= s >> 27;
  return s * 0x2545F4914F6CDD1Dull;
}

int main(int argc, char** argv) {
  const long n_random = argc > 1 ? atol(argv[1]) : 100000;
  std::vector<double> v;
  const double base[] = {0.0, 4.9406564584124654e-324, DBL_MIN, 1e-300, 0.2, 1.0, 10.0, 1e300, DBL_MAX, INFINITY,
                         0.5, 3.0, 2.220446049250313e-15};
  for (double b : base) {
    for (double x : {b, nextafter(b, INFINITY), nextafter(b, 0.0)}) {
      v.push_back(x);
      v.push_back(-x);
    }
  }
  for (uint64_t nan : {0x7FF8000000000000ull, 0x7FF0000000000001ull, 0x7FFFFFFFFFFFFFFFull, 0x7FF4000000000000ull}) {
    v.push_back(from_bits(nan));
    v.push_back(from_bits(nan | 0x8000000000000000ull));
  }
  const size_t n_special = v.size();
  for (long i = 0; i < n_random; ++i) v.push_back(from_bits(rnd()));
  // random patterns near the constants and zero
  for (long i = 0; i < n_random; ++i) {
    const double c = base[rnd() % (sizeof(base) / sizeof(base[0]))];
    uint64_t b;
    memcpy(&b, &c, 8);
    b += (rnd() % 65) - 32;
    if (rnd() & 1) b ^= 0x8000000000000000ull;
    v.push_back(from_bits(b));
  }

  const double consts[] = {0.2, 1.0, 10.0, 1e300, INFINITY, DBL_MIN, 4.9406564584124654e-324, DBL_MAX, 0.5};
  long checks = 0, bad = 0;
  auto expect = [&](bool got, bool want) {
    ++checks;
    if (got != want) ++bad;
  };
  expect(hg_bits(0.2) == HG_BITS_0_2, true);
  expect(hg_bits(1.0) == HG_BITS_1, true);
  expect(hg_bits(10.0) == HG_BITS_10, true);
  expect(hg_bits(1e300) == HG_BITS_1E300, true);
  for (size_t i = 0; i < v.size(); ++i) {
    const double x = v[i];
    expect(hg_isnan_cmp(x), x != x);
    expect(hg_eq0(x), x == 0.0);
    expect(hg_gt0(x), x > 0.0);
    expect(hg_lt0(x), x < 0.0);
    expect(hg_in_open_pos(x, HG_BITS_1E300), x > 0.0 && x < 1e300);
    for (double c : consts) {
      const uint64_t cb = hg_bits(c);
      expect(hg_lt_pos(x, cb), x < c);
      expect(hg_le_pos(x, cb), x <= c);
      expect(hg_gt_pos(x, cb), x > c);
      expect(hg_lt_neg(x, hg_bits(-c)), x < -c);
    }
  }
  // pairs: every special value with every value, and random pairs
  for (size_t i = 0; i < n_special; ++i) {
    for (size_t j = 0; j < v.size(); ++j) {
      const double a = v[i], b = v[j];
      expect(hg_gt(a, b), a > b);
      expect(hg_gt(b, a), b > a);
      expect(hg_both0(a, b), a == 0.0 && b == 0.0);
    }
  }
  for (long i = 0; i < n_random; ++i) {
    const double a = v[rnd() % v.size()], b = v[rnd() % v.size()];
    expect(hg_gt(a, b), a > b);
    expect(hg_both0(a, b), a == 0.0 && b == 0.0);
  }
  printf("%ld %ld\n", checks, bad);
  return 0;
}
