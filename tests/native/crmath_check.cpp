// Host build of hiten_gb300/csrc/hg_crmath.cuh compared against quad-precision
// pow (rounded once) on random inputs.  Prints the mismatch counts.
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>
#include "hg_crmath.cuh"
#if defined(__aarch64__)
typedef long double q_t;
#define QPOW powl
#else
#include <quadmath.h>
typedef __float128 q_t;
#define QPOW powq
#endif

static uint64_t s = 0x9E3779B97F4A7C15ull;
static double urand() {  // xorshift64*
  s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
  return (double)((s * 0x2545F4914F6CDD1Dull) >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  long bad15 = 0, bad25 = 0, badp = 0;
  const double ys[4] = {-1.0 / 9.0, 0.4 * (1.0 / 9.0), -0.125, 0.3};
  for (long i = 0; i < n; ++i) {
    const double x = pow(10.0, -4.0 + 5.0 * urand());
    double a, b;
    hg_pow15_25(x, a, b);
    if (a != (double)QPOW((q_t)x, (q_t)1.5)) ++bad15;
    if (b != (double)QPOW((q_t)x, (q_t)2.5)) ++bad25;
    const double xe = pow(10.0, -30.0 + 33.0 * urand());
    const double y = ys[i & 3];
    if (hg_pow(xe, y) != (double)QPOW((q_t)xe, (q_t)y)) ++badp;
  }
  // binade edges over a wide exponent range: mantissas just below the next
  // power of two (the hard cases of x^1.5 near a rounding midpoint) and
  // just above a power of two
  for (long i = 0; i < n; ++i) {
    const uint64_t r = (uint64_t)(urand() * 9007199254740992.0);
    const int mode = (int)(i % 2);
    const uint64_t mant = mode == 0 ? 0x000FFFFFFFFFFFFFull - (r & 0xFF) : (r & 0xFF);
    const uint64_t e = 1023 + (r >> 8) % 601 - 300;
    const uint64_t bits = (e << 52) | mant;
    double x;
    memcpy(&x, &bits, 8);
    double a, b;
    hg_pow15_25(x, a, b);
    if (a != (double)QPOW((q_t)x, (q_t)1.5)) ++bad15;
    if (b != (double)QPOW((q_t)x, (q_t)2.5)) ++bad25;
  }
  printf("%ld %ld %ld %ld\n", n, bad15, bad25, badp);
  return 0;
}
