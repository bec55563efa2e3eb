// Host build of hg_log_dd / hg_exp_dd (hiten_gb300/csrc/hg_crmath.cuh), whose
// argument reduction runs on the integer pipes, against the same functions
// with the reduction in floating point (rint of (m - 1) * 1024, compares on
// doubles) written out below: both outputs must agree bit for bit on random
// positive doubles over the whole range, subnormals, the mantissas around
// sqrt(2) and every kind of rounding tie of the table index.  Prints the
// number of inputs and of mismatches.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "hg_crmath.cuh"

// the floating-point reduction
static void log_dd_fp(double x, double& Lh, double& Ll) {
  int e = 0;
  if (x < 2.2250738585072014e-308) {
    x *= 18014398509481984.0;
    e = -54;
  }
  const uint64_t b = hg_bits(x);
  e += (int)((b >> 52) & 0x7ff) - 1023;
  double m = hg_from_bits((b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);
  if (m > 1.4142135623730951) {
    m *= 0.5;
    e += 1;
  }
  const int j = (int)rint((m - 1.0) * 1024.0);
  const double F = 1.0 + (double)j * 0.0009765625;
  const double f = m - F;
  const int ti = j - HG_LOG_JMIN;
  const double invF = HG_TAB(log_invf, ti);
  const double vh = f * invF;
  const double vl = fma(-vh, F, f) * invF;
  double q, qe;
  hg_two_prod(vh, vh, q, qe);
  double S = -0.125;
  S = fma(S, vh, 0.14285714285714285);
  S = fma(S, vh, -0.16666666666666666);
  S = fma(S, vh, 0.2);
  S = fma(S, vh, -0.25);
  S = fma(S, vh, 0.3333333333333333);
  const double T = (q * vh) * S;
  double A, Ae;
  hg_two_sum(vh, -0.5 * q, A, Ae);
  const double Pl = Ae + (vl + ((-0.5 * qe - vh * vl) + T));
  const double a = (double)e * HG_LN2_HI;
  double s1, e1, s2, e2;
  hg_two_sum(a, HG_TAB(log_th, ti), s1, e1);
  hg_two_sum(s1, A, s2, e2);
  const double low = ((e1 + e2) + (HG_TAB(log_tl, ti) + Pl)) + (double)e * HG_LN2_LO;
  hg_fast_two_sum(s2, low, Lh, Ll);
}

static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t rnd() {  // xorshift64*
  s ^= s >> 12;
  s ^= s << 25;
  s ^= s >> 27;
  return s * 0x2545F4914F6CDD1Dull;
}

static long n_in = 0, bad = 0;
static void check_log(uint64_t bits) {
  const double x = hg_from_bits(bits);
  double a, b, c, d;
  hg_log_dd(x, a, b);
  log_dd_fp(x, c, d);
  ++n_in;
  if (hg_bits(a) != hg_bits(c) || hg_bits(b) != hg_bits(d)) ++bad;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  // random positive finite doubles (subnormals included)
  for (long i = 0; i < n; ++i) {
    const uint64_t b = rnd() % 0x7FF0000000000000ull;
    if (b) check_log(b);
  }
  // the exponent range of the step-size controller's errors
  for (long i = 0; i < n; ++i) {
    const uint64_t ex = 1023 - 60 + rnd() % 80;
    check_log((ex << 52) | (rnd() & 0x000FFFFFFFFFFFFFull));
  }
  // mantissas around sqrt(2) and the ends of the mantissa range
  for (long k = -4096; k <= 4096; ++k) {
    const uint64_t ex = (1023 - 30 + (uint64_t)(rnd() % 60)) << 52;
    check_log(ex | (uint64_t)(0x6A09E667F3BCDll + k));
    check_log(ex | (uint64_t)(k & 0xFFF));
    check_log(ex | (0x000FFFFFFFFFFFFFull - (uint64_t)(k & 0xFFF)));
  }
  // ties of the table index and their neighbours: the low 42 (unhalved) or
  // 43 (halved) mantissa bits at half, for even and odd quotients
  for (long i = 0; i < n / 4; ++i) {
    const int sh = (i & 1) ? 43 : 42;
    const uint64_t hi = rnd() & ((1ull << (52 - sh)) - 1ull);
    uint64_t M = (hi << sh) | (1ull << (sh - 1));
    M += (uint64_t)((long)(rnd() % 5) - 2);
    M &= 0x000FFFFFFFFFFFFFull;
    const uint64_t ex = (1023 - 40 + (uint64_t)(rnd() % 80)) << 52;
    check_log(ex | M);
    check_log((rnd() % 2047 + 1) << 52 | M);  // any exponent
    check_log(M ? M : 1);                     // subnormal
  }
  // exp guards: |th| around 85, signed zeros, infinities, NaN
  const double ths[] = {85.0, nextafter(85.0, 0.0), nextafter(85.0, 1e9), -85.0, nextafter(-85.0, 0.0),
                        nextafter(-85.0, -1e9), 0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, -NAN, 1e300};
  long n_exp = 0, bad_exp = 0;
  for (double th : ths) {
    ++n_exp;
    const double r = hg_exp_dd(th, 0.0);
    double want;
    if (th > 85.0)
      want = 8.0e36;
    else if (th < -85.0)
      want = 1.2e-37;
    else
      want = NAN;  // checked below: the guards must not fire
    if (th > 85.0 || th < -85.0) {
      if (hg_bits(r) != hg_bits(want)) ++bad_exp;
    } else if (r == 8.0e36 || r == 1.2e-37) {
      ++bad_exp;
    }
  }
  printf("%ld %ld %ld %ld\n", n_in, bad, n_exp, bad_exp);
  return 0;
}
