// Correctly rounded power functions in FP64 for the propagation kernels.
//
// The reference evaluates x**1.5, x**2.5 (CR3BP Jacobian, dynamics/rtbp.py:117-122,
// :232-235) and err**(-1/9), err**(0.4/9), err**(-1/8) (PI step-size
// controller, integrators/utils.py:218-296) with libm pow.  These kernels
// return the correctly rounded result (the exact power rounded once to
// nearest), which is what a perfect libm returns; libm itself misrounds
// about one call in a thousand.  The CPU oracle's DEVICE mode computes the same
// values in quad precision.
//
// Methods (all error-free transforms are Dekker/Knuth two-product and
// two-sum on fused multiply-add hardware):
//   * hg_pow15 / hg_pow25: x*sqrt(x) in double-double.  s = RN(sqrt(x)),
//     the residual x - s^2 is exact (fma), sqrt(x) = s + (x - s^2)/(2s) to
//     ~2^-104, and x*s is split exactly; total error ~2^-100 before the
//     final rounding.  (hg_pow15_25 on the device: the same split from a
//     Goldschmidt square root, see there.)
//   * hg_pow: exp(y * log(x)).  log by Tang's table method (F_j = 1+j/1024,
//     log(1+v) series, v = (m-F)/F in double-double), exp by Tang's table
//     method (2^(j/256) in double-double, Cody-Waite reduction with ln2/256
//     split in three parts, Taylor polynomial for exp(r)-1).  Relative
//     error before the final rounding is ~2^-83 for |y log x| <= 85.
//
// The header compiles as device code (nvcc) and as host C++ (g++ with
// -ffp-contract=off) so the same arithmetic can be unit-tested on the CPU.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "hg_crmath_tables.h"

#if defined(__CUDACC__)
#define HG_HD __host__ __device__ __forceinline__
#else
#define HG_HD static inline
#endif

#if defined(__CUDACC__)
__device__ static const double hg_d_log_invf[HG_LOG_N] = HG_LOG_INVF_INIT;
__device__ static const double hg_d_log_th[HG_LOG_N] = HG_LOG_TH_INIT;
__device__ static const double hg_d_log_tl[HG_LOG_N] = HG_LOG_TL_INIT;
__device__ static const double hg_d_exp_th[256] = HG_EXP_TH_INIT;
__device__ static const double hg_d_exp_tl[256] = HG_EXP_TL_INIT;
#endif
static const double hg_h_log_invf[HG_LOG_N] = HG_LOG_INVF_INIT;
static const double hg_h_log_th[HG_LOG_N] = HG_LOG_TH_INIT;
static const double hg_h_log_tl[HG_LOG_N] = HG_LOG_TL_INIT;
static const double hg_h_exp_th[256] = HG_EXP_TH_INIT;
static const double hg_h_exp_tl[256] = HG_EXP_TL_INIT;

#if defined(__CUDA_ARCH__)
#define HG_TAB(name, i) __ldg(&hg_d_##name[i])
#else
#define HG_TAB(name, i) (hg_h_##name[i])
#endif

HG_HD uint64_t hg_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}

HG_HD double hg_from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}

HG_HD double hg_rsqrt_approx(double x) {
#if defined(__CUDA_ARCH__)
  return rsqrt(x);
#else
  return 1.0 / sqrt(x);
#endif
}

HG_HD void hg_two_prod(double a, double b, double& p, double& e) {
  p = a * b;
  e = fma(a, b, -p);
}

HG_HD void hg_two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

HG_HD void hg_fast_two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  e = b - (s - a);
}

// ---------------------------------------------------------------------------
// IEEE comparisons on the integer pipes.  In the propagation kernels the SM's
// FP64 unit is the bottleneck and a floating-point compare takes a slot of it;
// these compare bit patterns (hg_bits) instead and equal the IEEE comparison
// for every operand (a NaN compares false, -0 equals +0).  Non-negative
// doubles order like their bit patterns read as integers.
// ---------------------------------------------------------------------------
static const uint64_t HG_BITS_INF = 0x7FF0000000000000ull;
static const uint64_t HG_BITS_NEG_INF = 0xFFF0000000000000ull;

HG_HD bool hg_isnan_cmp(double x) { return (hg_bits(x) << 1) > (HG_BITS_INF << 1); }
// x == 0
HG_HD bool hg_eq0(double x) { return (hg_bits(x) << 1) == 0; }
// x == 0 && y == 0
HG_HD bool hg_both0(double x, double y) { return ((hg_bits(x) | hg_bits(y)) << 1) == 0; }
// x > 0: the patterns of +denorm_min .. +inf
HG_HD bool hg_gt0(double x) { return hg_bits(x) - 1ull < HG_BITS_INF; }
// x < 0: the patterns of -denorm_min .. -inf
HG_HD bool hg_lt0(double x) { return hg_bits(x) - 0x8000000000000001ull < HG_BITS_INF; }
// 0 < x < c for c > 0 given by its pattern cb (c not NaN)
HG_HD bool hg_in_open_pos(double x, uint64_t cb) { return hg_bits(x) - 1ull < cb - 1ull; }
// x < c, x <= c and x > c for c > 0 given by its pattern cb (c may be +inf,
// not NaN): a negative x (any pattern with the sign set but a NaN's) is below c
HG_HD bool hg_lt_pos(double x, uint64_t cb) {
  const uint64_t b = hg_bits(x);
  return (int64_t)b < (int64_t)cb && b <= HG_BITS_NEG_INF;
}
HG_HD bool hg_le_pos(double x, uint64_t cb) {
  const uint64_t b = hg_bits(x);
  return (int64_t)b <= (int64_t)cb && b <= HG_BITS_NEG_INF;
}
HG_HD bool hg_gt_pos(double x, uint64_t cb) {
  const uint64_t b = hg_bits(x);
  return (int64_t)b > (int64_t)cb && (int64_t)b <= (int64_t)HG_BITS_INF;
}
// x < c for c < 0 given by its pattern cb (c not NaN): x is negative with a
// larger magnitude pattern, and not a NaN
HG_HD bool hg_lt_neg(double x, uint64_t cb) {
  const uint64_t b = hg_bits(x);
  return b > cb && b <= HG_BITS_NEG_INF;
}
// a > b for any a, b: the sign-magnitude patterns mapped to ordered
// two's-complement keys (-0 and +0 to the same key 0)
HG_HD int64_t hg_order_key(uint64_t b) {
  const int64_t m = (int64_t)(b & 0x7FFFFFFFFFFFFFFFull);
  return (int64_t)b < 0 ? -m : m;
}
HG_HD bool hg_gt(double a, double b) {
  return !hg_isnan_cmp(a) && !hg_isnan_cmp(b) && hg_order_key(hg_bits(a)) > hg_order_key(hg_bits(b));
}
// patterns of the constants the step control compares with
static const uint64_t HG_BITS_0_2 = 0x3FC999999999999Aull;    // 0.2
static const uint64_t HG_BITS_1 = 0x3FF0000000000000ull;      // 1.0
static const uint64_t HG_BITS_10 = 0x4024000000000000ull;     // 10.0
static const uint64_t HG_BITS_1E300 = 0x7E37E43C8800759Cull;  // 1e300

// Correctly rounded quotient a / b from the correctly rounded reciprocal
// rb = RN(1/b) (Markstein's theorem, IBM J. Res. Dev. 34(1), 1990; see also
// the Handbook of Floating-Point Arithmetic, sec. 4.7): q0 = RN(a*rb) is
// within one ulp of a/b, the remainder r = a - b*q0 is exact with an fma,
// and RN(q0 + r*rb) = RN(a/b).  Valid for finite, normal operands whose
// quotient and remainder neither overflow nor underflow -- the CR3BP values
// on this path (distances 1e-3..1e3) stay far from those limits.  A zero
// numerator (z = 0 in a planar problem) gives a zero quotient whose sign can
// differ from IEEE division's (+0 for -0 / b); keeping that sign costs 2-6 %
// of the propagation kernels' time, so it is not kept.  One reciprocal
// serves every quotient with the same denominator: 3 FP64 operations per
// quotient instead of a full division.
HG_HD double hg_div_rn(double a, double b, double rb) {
  const double q0 = a * rb;
  const double r = fma(-b, q0, a);
  return fma(r, rb, q0);
}

HG_HD double hg_rcp_rn(double b) {
#if defined(__CUDA_ARCH__)
  return __drcp_rn(b);
#else
  return 1.0 / b;
#endif
}

// x^1.5 as an unevaluated sum hi + lo (|lo| <= ~1.5 ulp(hi)), x > 0 normal.
HG_HD void hg_pow15_dd(double x, double& hi, double& lo) {
  const double s = sqrt(x);
  const double rho = fma(-s, s, x);              // exact residual x - s^2
  const double d = rho * (0.5 * hg_rsqrt_approx(x));  // sqrt(x) - s to ~2^-50 relative
  hi = x * s;
  lo = fma(x, s, -hi);
  lo = fma(x, d, lo);
}

HG_HD double hg_pow15(double x) {
  if (!(x > 0.0) || !(x < 1e300) || x < 1e-290) return pow(x, 1.5);
  double hi, lo;
  hg_pow15_dd(x, hi, lo);
  return hi + lo;
}

// Both x^1.5 and x^2.5 (shared square root).
//
// Device: the range test runs on the integer pipe (exponent field of x in
// [625, 1421], i.e. 2^-398 <= x < 2^399, sign clear), and sqrt(x) as
// g + e comes from Goldschmidt's coupled iteration (g -> sqrt(x),
// h -> 1/(2 sqrt(x)); P. Markstein, "Software division and square root
// using Goldschmidt's algorithms", 6th Conf. on Real Numbers and Computers,
// 2004) seeded by the hardware reciprocal-square-root estimate (PTX
// rsqrt.approx.f64, ~2^-22 relative): two iterations bring g and h to
// rounding level, the residual d = x - g^2 (one fma) gives e = d h, and
// x (g + e) is split exactly as on the host: ~2^-102 relative error before
// the final rounding, 10 FP64 operations for the square root instead of a
// correctly rounded sqrt plus a reciprocal square root.  Host: the
// sqrt-based double-double of hg_pow15_dd.
HG_HD void hg_pow15_25(double x, double& p15, double& p25) {
#if defined(__CUDA_ARCH__)
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  if ((unsigned)(bits >> 52) - 625u > 796u) {
    p15 = pow(x, 1.5);
    p25 = pow(x, 2.5);
    return;
  }
  double y0;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(y0) : "d"(x));
  double g = x * y0, h = 0.5 * y0;
  double r = fma(-g, h, 0.5);
  g = fma(g, r, g);
  h = fma(h, r, h);
  r = fma(-g, h, 0.5);
  g = fma(g, r, g);
  h = fma(h, r, h);
  const double e = fma(-g, g, x) * h;
  const double hi = x * g;
  double lo = fma(x, g, -hi);
  lo = fma(x, e, lo);
#else
  if (!(x > 0.0) || !(x < 1e120) || x < 1e-120) {
    p15 = pow(x, 1.5);
    p25 = pow(x, 2.5);
    return;
  }
  double hi, lo;
  hg_pow15_dd(x, hi, lo);
#endif
  p15 = hi + lo;
  const double h2 = x * hi;
  double l2 = fma(x, hi, -h2);
  l2 = fma(x, lo, l2);
  p25 = h2 + l2;
  // The one family of hard cases the double-double cannot resolve:
  // x = 2^(2q) (1 - 2^-53) (mantissa all ones, even biased exponent), where
  // x^1.5 = 2^(3q) (1 - 1.5 u + 0.375 u^2 + ...) lies 0.375 u^2 (u = 2^-53)
  // above a rounding midpoint.  Exactly: RN(x^1.5) = 2^(3q) (1 - u),
  // RN(x^2.5) = 2^(5q) (1 - 2u).
  const uint64_t b = hg_bits(x);
  if ((b & 0x000FFFFFFFFFFFFFull) == 0x000FFFFFFFFFFFFFull && ((b >> 52) & 1u) == 0) {
    const int q = ((int)(b >> 52) - 1022) / 2;
    p15 = hg_from_bits(((uint64_t)(3 * q + 1022) << 52) | 0x000FFFFFFFFFFFFFull);
    p25 = hg_from_bits(((uint64_t)(5 * q + 1022) << 52) | 0x000FFFFFFFFFFFFEull);
  }
}

// One of the two powers: RN(x^1.5) when !want25, RN(x^2.5) when want25 --
// the bits hg_pow15_25 gives.  For lanes of a warp that want different
// ones: the final sum hi + lo of x^1.5 and the leading product RN(x * hi) of
// x^2.5 share one fused multiply-add (fma(1, hi, lo) = RN(hi + lo),
// fma(x, hi, 0) = RN(x hi) for x hi > 0), one FP64 instruction fewer than
// forming both.
HG_HD double hg_pow15_or_25(double x, bool want25) {
#if defined(__CUDA_ARCH__)
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  if ((unsigned)(bits >> 52) - 625u > 796u) return pow(x, want25 ? 2.5 : 1.5);
  double y0;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(y0) : "d"(x));
  double g = x * y0, h = 0.5 * y0;
  double r = fma(-g, h, 0.5);
  g = fma(g, r, g);
  h = fma(h, r, h);
  r = fma(-g, h, 0.5);
  g = fma(g, r, g);
  h = fma(h, r, h);
  const double e = fma(-g, g, x) * h;
  const double hi = x * g;
  double lo = fma(x, g, -hi);
  lo = fma(x, e, lo);
  const double f = fma(want25 ? x : 1.0, hi, want25 ? 0.0 : lo);  // hi + lo | RN(x hi)
  double l2 = fma(x, hi, -f);
  l2 = fma(x, lo, l2);
  double p = want25 ? f + l2 : f;
  const uint64_t b = bits;
  if ((b & 0x000FFFFFFFFFFFFFull) == 0x000FFFFFFFFFFFFFull && ((b >> 52) & 1u) == 0) {
    const int q = ((int)(b >> 52) - 1022) / 2;
    p = want25 ? hg_from_bits(((uint64_t)(5 * q + 1022) << 52) | 0x000FFFFFFFFFFFFEull)
               : hg_from_bits(((uint64_t)(3 * q + 1022) << 52) | 0x000FFFFFFFFFFFFFull);
  }
  return p;
#else
  double p15, p25;
  hg_pow15_25(x, p15, p25);
  return want25 ? p25 : p15;
#endif
}

// log(x) as double-double, x > 0 finite.  Absolute error <~ 2^-85.
// The reduction x = 2^e m, m in (sqrt(2)/2, sqrt(2)], and the table index
// j = rint((m - 1) * 1024) with F = 1 + j / 1024 are formed from the bit
// pattern on the integer pipes: for m = 1 + M 2^-52 (M the mantissa field),
// (m - 1) * 1024 = M 2^-42; for m = (1 + M 2^-52) / 2 it is M 2^-43 - 512; the
// shift rounds half to even as rint does, and F's pattern is 1.0's plus
// j 2^42 (j >= 0) or minus |j| 2^43 (j < 0, F in [1/2, 1)).  Every value is
// the one the floating-point reduction gives.
HG_HD void hg_log_dd(double x, double& Lh, double& Ll) {
  int e = 0;
  if (hg_lt_pos(x, 0x0010000000000000ull)) {  // x < 2^-1022 (subnormal)
    x *= 18014398509481984.0;                  // 2^54
    e = -54;
  }
  const uint64_t b = hg_bits(x);
  const uint64_t M = b & 0x000FFFFFFFFFFFFFull;
  const bool halve = M > 0x6A09E667F3BCDull;  // 1 + M 2^-52 > 1.4142135623730951
  e += (int)((b >> 52) & 0x7ff) - 1023 + (halve ? 1 : 0);
  const double m = hg_from_bits(M | (halve ? 0x3FE0000000000000ull : 0x3FF0000000000000ull));
  const int sh = halve ? 43 : 42;
  const uint64_t jq = M >> sh;
  const uint64_t jr = M & ((1ull << sh) - 1ull);
  const uint64_t jh = 1ull << (sh - 1);
  const int j = (int)(jq + ((jr > jh || (jr == jh && (jq & 1ull))) ? 1ull : 0ull)) - (halve ? 512 : 0);
  const double F = hg_from_bits(j >= 0 ? 0x3FF0000000000000ull + ((uint64_t)j << 42)
                                       : 0x3FF0000000000000ull - ((uint64_t)(-j) << 43));
  const double f = m - F;  // exact (Sterbenz)
  const int ti = j - HG_LOG_JMIN;
  const double invF = HG_TAB(log_invf, ti);
  const double vh = f * invF;
  const double vl = fma(-vh, F, f) * invF;  // v = vh + vl = f/F to ~2^-104
  // log(1+v) = v - v^2/2 + v^3 * S(v)
  double q, qe;
  hg_two_prod(vh, vh, q, qe);
  double S = -0.125;                         // -1/8
  S = fma(S, vh, 0.14285714285714285);       // 1/7
  S = fma(S, vh, -0.16666666666666666);      // -1/6
  S = fma(S, vh, 0.2);                       // 1/5
  S = fma(S, vh, -0.25);                     // -1/4
  S = fma(S, vh, 0.3333333333333333);        // 1/3
  // 1/3 etc. are rounded; their error (2^-55 relative) times v^3 (<2^-31)
  // stays below 2^-86.
  const double T = (q * vh) * S;
  double A, Ae;
  hg_two_sum(vh, -0.5 * q, A, Ae);
  const double Pl = Ae + (vl + ((-0.5 * qe - vh * vl) + T));
  // L = e*ln2 + log(F) + (A + Pl)
  const double a = (double)e * HG_LN2_HI;  // exact (40-bit constant)
  double s1, e1, s2, e2;
  hg_two_sum(a, HG_TAB(log_th, ti), s1, e1);
  hg_two_sum(s1, A, s2, e2);
  const double low = ((e1 + e2) + (HG_TAB(log_tl, ti) + Pl)) + (double)e * HG_LN2_LO;
  hg_fast_two_sum(s2, low, Lh, Ll);
}

// exp(th + tl), |th| <= 85, correctly rounded except with probability ~2^-29.
HG_HD double hg_exp_dd(double th, double tl) {
  if (hg_gt_pos(th, 0x4055400000000000ull)) return 8.0e36;   // th > 85
  if (hg_lt_neg(th, 0xC055400000000000ull)) return 1.2e-37;  // th < -85
  const double kd = rint(th * HG_INV_L256);
  const int k = (int)kd;
  const double r0 = th - kd * HG_L256_1;  // exact (Sterbenz, 38-bit constant)
  double r1, r1e;
  hg_two_sum(r0, -kd * HG_L256_2, r1, r1e);  // kd*L2 exact (38-bit constant)
  double rh, rl;
  hg_fast_two_sum(r1, (r1e + tl) - kd * HG_L256_3, rh, rl);
  // exp(r) - 1 = r + r^2/2 + r^3 * S(r),  |r| <= ln2/512
  double q, qe;
  hg_two_prod(rh, rh, q, qe);
  double S = 1.3888888888888889e-03;          // 1/720
  S = fma(S, rh, 8.3333333333333332e-03);     // 1/120
  S = fma(S, rh, 4.1666666666666664e-02);     // 1/24
  S = fma(S, rh, 1.6666666666666666e-01);     // 1/6
  const double T = (q * rh) * S;
  double E, Ee;
  hg_two_sum(rh, 0.5 * q, E, Ee);
  const double El = Ee + (rl + ((0.5 * qe + rh * rl) + T));
  // 2^(j/256) * (1 + E + El)
  const int jj = k & 255;
  const int sh = (k - jj) / 256;
  const double Th = HG_TAB(exp_th, jj);
  const double Tl = HG_TAB(exp_tl, jj);
  double ph, pe;
  hg_two_prod(Th, E, ph, pe);
  const double cl = ((pe + Th * El) + Tl) + Tl * E;
  double s, se;
  hg_two_sum(Th, ph, s, se);
  const double res = s + (se + cl);
  // scale by 2^sh (|sh| <= 123: exact power of two, result stays normal)
  return res * hg_from_bits((uint64_t)(sh + 1023) << 52);
}

// Correctly rounded x^y for x > 0 finite and |y log x| <= 85; other inputs
// fall back to the platform pow (never reached by the step-size controller
// for finite errors, where the result is clamped anyway).
HG_HD double hg_pow(double x, double y) {
  if (!(x > 0.0) || !(x < 1.0e308) || !(y == y)) return pow(x, y);
  if (x == 1.0 || y == 0.0) return 1.0;
  double Lh, Ll;
  hg_log_dd(x, Lh, Ll);
  double th, pe;
  hg_two_prod(y, Lh, th, pe);
  const double tl = fma(y, Ll, pe);
  double Th, Tl;
  hg_fast_two_sum(th, tl, Th, Tl);
  return hg_exp_dd(Th, Tl);
}
