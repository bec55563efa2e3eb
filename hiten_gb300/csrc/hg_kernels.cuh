// sm_103a kernels for the CR3BP propagation path (FP64 throughout).
//
// Execution model.  GB300 issues FP64 at a small fraction of its FP32 rate,
// so the kernels are bound by the FP64 pipe, not by HBM: state and Runge-
// Kutta stages live in registers, HBM sees only initial states, sampled
// outputs and saved event steps.  Lane layouts (Layout<G>):
//   * G = 1  (6-dim state): one lane owns one trajectory.
//   * G = 2  (6-dim): a lane pair (position / velocity halves).
//   * G = 6  (6-dim): six lanes, one component each.
//   * G = 7  (42-dim state + STM): a group of 7 lanes owns one trajectory;
//            lane j < 6 holds STM column j (components 6r+j, r = 0..5), lane 6
//            holds the state (components 36..41).  Column j of dPhi = F(x)Phi
//            needs only the state, which the state lane broadcasts by shuffle
//            at every stage; the group shares the Hessian's work.  Four
//            groups fill lanes 0..27.
// Wider groups cut the per-step latency of one trajectory (what bounds a
// batch whose longest trajectories run alone at the end); narrower ones
// spend the least FP64 work per step.
// Group-wide decisions (accept/reject, events) use values that every lane of
// the group computes identically, so control flow stays group-uniform.
//
// Arithmetic follows the reference's expression order exactly (no
// contraction: the library is built with --fmad=false; fma appears only in
// explicit error-free transforms and in the numpy-dot order), so results are
// bit-identical to the CPU oracle's DEVICE mode.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>
#include <utility>

#include "hg_crmath.cuh"
#include "hg_tableaux.h"
#include "hitengpu.h"

namespace hg {

template <int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  [&]<int... I>(std::integer_sequence<int, I...>) {
    (f(std::integral_constant<int, I>{}), ...);
  }(std::make_integer_sequence<int, N>{});
}

// ---------------------------------------------------------------------------
// Fixed-step tableaux (integrators/coefficients/{rk4,rk6,rk8}.py)
// ---------------------------------------------------------------------------
template <int ORDER>
struct FixedTab;
template <>
struct FixedTab<4> {
  static constexpr int S = 4;
  __host__ __device__ static constexpr double a(int i, int j) { return HG_RK4_A[i][j]; }
  __host__ __device__ static constexpr double b(int j) { return HG_RK4_B[j]; }
};
template <>
struct FixedTab<6> {
  static constexpr int S = 7;
  __host__ __device__ static constexpr double a(int i, int j) { return HG_RK6_A[i][j]; }
  __host__ __device__ static constexpr double b(int j) { return HG_RK6_B[j]; }
};
template <>
struct FixedTab<8> {
  static constexpr int S = 13;
  __host__ __device__ static constexpr double a(int i, int j) { return HG_RK8_A[i][j]; }
  __host__ __device__ static constexpr double b(int j) { return HG_RK8_B[j]; }
};

// DOP853 (integrators/coefficients/dop853.py): A[:12,:12], B = A[12,:12],
// E5/E3 over 13 stages, extended rows 13..15 and D for dense output.
struct DopTab {
  static constexpr int S = HG_DOP_N_STAGES;       // 12
  static constexpr int SE = HG_DOP_N_STAGES_EXT;  // 16
  static constexpr int IP = HG_DOP_INTERP_POWER;  // 7
  __host__ __device__ static constexpr double a(int i, int j) { return HG_DOP_A[i][j]; }
  __host__ __device__ static constexpr double b(int j) { return HG_DOP_B[j]; }
  __host__ __device__ static constexpr double e5(int j) { return HG_DOP_E5[j]; }
  __host__ __device__ static constexpr double e3(int j) { return HG_DOP_E3[j]; }
  __host__ __device__ static constexpr double d(int i, int j) { return HG_DOP_D[i][j]; }
};

// ---------------------------------------------------------------------------
// Vector fields
// ---------------------------------------------------------------------------

// dynamics/rtbp.py:30-74 (_crtbp_accel), numba lowering of ** (x*x, x*(x*x)).
// The six quotients share the two denominators r1^3 and r2^3: each is the
// correctly rounded quotient (hg_div_rn), i.e. the same bits as `/`.
__device__ __forceinline__ void rhs6(const double (&s)[6], double mu, double (&d)[6]) {
  const double x = s[0], y = s[1], z = s[2], vx = s[3], vy = s[4];
  const double omu = 1.0 - mu;
  const double t1 = x + mu;
  const double yy = y * y;
  const double zz = z * z;
  const double r1 = sqrt((t1 * t1 + yy) + zz);
  const double t2 = x - omu;
  const double r2 = sqrt((t2 * t2 + yy) + zz);
  const double r1c = r1 * (r1 * r1);
  const double r2c = r2 * (r2 * r2);
  const double i1 = hg_rcp_rn(r1c);
  const double i2 = hg_rcp_rn(r2c);
  d[0] = vx;
  d[1] = vy;
  d[2] = s[5];
  d[3] = ((2.0 * vy + x) - hg_div_rn(omu * t1, r1c, i1)) - hg_div_rn(mu * ((x - 1.0) + mu), r2c, i2);
  d[4] = ((-2.0 * vx + y) - hg_div_rn(omu * y, r1c, i1)) - hg_div_rn(mu * y, r2c, i2);
  d[5] = hg_div_rn((-omu) * z, r1c, i1) - hg_div_rn(mu * z, r2c, i2);
}

// Hessian of the effective potential and the state accelerations,
// dynamics/rtbp.py:76-165 and :215-238.
struct Hess {
  double xx, yy, zz, xy, xz, yz;
  double ax, ay, az;
};

__device__ __forceinline__ Hess hessian42(double x, double y, double z, double vx, double vy, double mu) {
  Hess H;
  const double mu2 = 1.0 - mu;
  const double t1 = x + mu;
  const double t2 = x - mu2;
  const double ys = y * y;
  const double zs = z * z;
  const double t1s = t1 * t1;
  const double t2s = t2 * t2;
  const double r2 = (t1s + ys) + zs;
  const double R2 = (t2s + ys) + zs;
  double r3, r5, R3, R5;
  hg_pow15_25(r2, r3, r5);
  hg_pow15_25(R2, R3, R5);
  const double i_r3 = hg_rcp_rn(r3), i_r5 = hg_rcp_rn(r5), i_R3 = hg_rcp_rn(R3), i_R5 = hg_rcp_rn(R5);
  const double qa = hg_div_rn(mu2, r5, i_r5);
  const double qb = hg_div_rn(mu, R5, i_R5);
  const double c3 = hg_div_rn(mu2, r3, i_r3) + hg_div_rn(mu, R3, i_R3);
  const double a3 = qa * 3.0;
  const double b3 = qb * 3.0;
  H.xx = ((1.0 + a3 * t1s) + b3 * t2s) - c3;
  H.yy = ((1.0 + a3 * ys) + b3 * ys) - c3;
  H.zz = (a3 * zs + b3 * zs) - c3;
  const double sxy = hg_div_rn(mu2 * t1, r5, i_r5) + hg_div_rn(mu * t2, R5, i_R5);
  H.xy = (3.0 * y) * sxy;
  H.xz = (3.0 * z) * sxy;
  H.yz = ((3.0 * y) * z) * (qa + qb);
  H.ax = ((x - mu2 * hg_div_rn(t1, r3, i_r3)) - mu * hg_div_rn(t2, R3, i_R3)) + 2.0 * vy;
  H.ay = ((y - mu2 * hg_div_rn(y, r3, i_r3)) - mu * hg_div_rn(y, R3, i_R3)) - 2.0 * vx;
  H.az = (-mu2) * hg_div_rn(z, r3, i_r3) - mu * hg_div_rn(z, R3, i_R3);
  return H;
}

// ---------------------------------------------------------------------------
// Lane layout
// ---------------------------------------------------------------------------
struct Dir {
  int neg_lo, neg_hi;  // component range whose derivative is negated (fwd=-1)
};

// -v when neg: the sign-bit flip IEEE negation is, on the integer pipe (the
// FP64 pipe is the scarce one).
__device__ __forceinline__ double neg_if(double v, bool neg) {
  return __longlong_as_double(__double_as_longlong(v) ^ (neg ? (long long)0x8000000000000000ull : 0ll));
}

template <int G>
struct Layout;

template <>
struct Layout<1> {
  static constexpr int D = 6;
  static constexpr int NC = 6;    // components per lane
  static constexpr int TPW = 32;  // trajectories per warp
  __device__ __forceinline__ int owner(int c) const { return 0; }
  __device__ __forceinline__ int local(int c) const { return c; }
  int role;                       // always 6 ("state" lane of a 6-dim system)
  __device__ __forceinline__ int comp(int r) const { return r; }
  __device__ __forceinline__ void rhs(const double (&v)[6], double mu, const Dir& dir, double (&dv)[6]) const {
    rhs6(v, mu, dv);
#pragma unroll
    for (int r = 0; r < 6; ++r)
      dv[r] = neg_if(dv[r], r >= dir.neg_lo && r < dir.neg_hi);
  }
  template <typename T>
  __device__ __forceinline__ T from_state(T v) const { return v; }
};

// hessian42 with its work spread over a lane group: lane base + job does job
// (0..5); L.from(v, r) reads lane base + r.  Lane b*3 + k (b = primary,
// k < 3) takes the power of its primary its quotients divide by (r^3 for
// k < 2, r^5 for k = 2; hg_pow15_or_25), one reciprocal and two of the
// twelve quotients:
//   0: mu2/r3, t1/r3     1: y/r3, z/r3     2: mu2/r5, (mu2 t1)/r5
//   3: mu/R3,  t2/R3     4: y/R3, z/R3     5: mu/R5,  (mu t2)/R5
// (further lanes repeat job 0).  The quotients are exchanged, lanes 0..5
// form xx, yy, zz, ax, ay, az with one common expression
// ((p + a u) + b w) + c whose operands reproduce hessian42's exactly
// (x - m == x + (-m), (-a) u == -(a u), -0 + v == v), and those six are
// exchanged again.  Same operations on the same operands: same bits.
// With OFFDIAG = false each of lanes 3..5 forms one off-diagonal entry, in
// H.xy: job 3 xy, job 4 yz, job 5 xz (the products below, their factors
// formed in the instructions that give lanes 0..2 b3 and c3).
template <class LT, bool OFFDIAG = true>
__device__ __forceinline__ Hess hessian_split(const LT& L, int job, double x, double y, double z, double vx, double vy,
                                            double mu) {
  const double mu2 = 1.0 - mu;
  const bool b2 = job >= 3;
  const int k = b2 ? job - 3 : job;
  const double m = b2 ? mu : mu2;
  // this lane's primary: tt = x + mu | x - mu2 (x - m == x + (-m))
  const double tt = x + (b2 ? -mu2 : mu);
  // the four squares and both numerators m tt in one multiply (job 0: t1^2,
  // 1: y^2, 2: mu2 t1, 3: t2^2, 4: z^2, 5: mu t2; further jobs repeat
  // job 0), the squares gathered from their lanes
  const double sq = (k == 0 ? tt : (job == 1 ? y : (job == 4 ? z : m))) * (job == 1 ? y : (job == 4 ? z : tt));
  const double t1s = L.from(sq, 0);
  const double t2s = L.from(sq, 3);
  const double ys = L.from(sq, 1);
  const double zs = L.from(sq, 4);
  const double rr = ((b2 ? t2s : t1s) + ys) + zs;
  const double den = hg_pow15_or_25(rr, k == 2);  // r^3 (jobs 0, 1) or r^5 (job 2) of the lane's primary
  const double inv = hg_rcp_rn(den);
  const double mt = sq;  // jobs 2 and 5
  const double n0 = k == 1 ? y : m;
  const double n1 = k == 0 ? tt : (k == 1 ? z : mt);
  const double q0 = hg_div_rn(n0, den, inv);
  const double q1 = hg_div_rn(n1, den, inv);
  // exchange: qa, qb, the r^3 terms of c3, the r^5 terms of sxy
  const double qa = L.from(q0, 2), qb = L.from(q0, 5);
  const double c3a = L.from(q0, 0), c3b = L.from(q0, 3);
  const double sxa = L.from(q1, 2), sxb = L.from(q1, 5);
  // acceleration lanes 3/4/5 read the x/y/z quotients of both primaries
  const int ua = job == 3 ? 0 : 1, wa = job == 3 ? 3 : 4;
  const double u0 = L.from(q0, ua), u1 = L.from(q1, ua), w0 = L.from(q0, wa), w1 = L.from(q1, wa);
  // job 0 xx, 1 yy, 2 zz, 3 ax, 4 ay, 5 az
  const bool acc = b2;
  const int e = job;
  // one multiply forms a3 = qa * 3 on jobs 0..2 and the Coriolis term
  // 2 vy / -2 vx on jobs 3, 4
  const double f1 = (acc ? (e == 4 ? -2.0 : 2.0) : qa) * (acc ? (e == 4 ? vx : vy) : 3.0);
  double b3, c3, f3 = 0.0, s2 = 0.0;
  if constexpr (OFFDIAG) {
    b3 = qb * 3.0;
    c3 = c3a + c3b;
  } else {
    // jobs 0..2 form b3 = qb * 3 and c3, jobs 3..5 the first factor of their
    // off-diagonal entry (3y or 3z) and its sum (sxy, or qa + qb for yz), in
    // the same two instructions
    f3 = (acc ? (e == 5 ? z : y) : qb) * 3.0;
    s2 = (acc ? (e == 4 ? qa : sxa) : c3a) + (acc ? (e == 4 ? qb : sxb) : c3b);
    b3 = f3;
    c3 = s2;
  }
  double P, A, U, B, W, Cc;
  if (!acc) {
    P = e == 2 ? -0.0 : 1.0;
    A = f1;
    U = e == 0 ? t1s : (e == 1 ? ys : zs);
    B = b3;
    W = e == 0 ? t2s : (e == 1 ? ys : zs);
    Cc = -c3;
  } else {
    P = e == 3 ? x : (e == 4 ? y : -0.0);
    A = -mu2;
    U = e == 3 ? u1 : (e == 4 ? u0 : u1);  // t1/r3 | y/r3 | z/r3
    B = -mu;
    W = e == 3 ? w1 : (e == 4 ? w0 : w1);  // t2/R3 | y/R3 | z/R3
    Cc = e == 5 ? -0.0 : f1;
  }
  const double form = ((P + A * U) + B * W) + Cc;
  Hess H;
  H.xx = L.from(form, 0);
  H.yy = L.from(form, 1);
  H.zz = L.from(form, 2);
  H.ax = L.from(form, 3);
  H.ay = L.from(form, 4);
  H.az = L.from(form, 5);
  if constexpr (OFFDIAG) {
    const double sxy = sxa + sxb;
    H.xy = (3.0 * y) * sxy;
    H.xz = (3.0 * z) * sxy;
    H.yz = ((3.0 * y) * z) * (qa + qb);
  } else {
    // this lane's off-diagonal entry as hessian42 forms it: job 3 xy = (3y) sxy,
    // job 4 yz = ((3y) z)(qa + qb), job 5 xz = (3z) sxy, one product
    // ((3a) b) c (c = 1.0 where two factors suffice: exact)
    H.xy = (f3 * (e == 4 ? z : s2)) * (e == 4 ? s2 : 1.0);
    H.xz = 0.0;
    H.yz = 0.0;
  }
  return H;
}

template <>
struct Layout<7> {
  static constexpr int D = 42;
  static constexpr int NC = 6;
  static constexpr int TPW = 4;
  __device__ __forceinline__ int owner(int c) const { return c >= 36 ? 6 : c % 6; }
  __device__ __forceinline__ int local(int c) const { return c >= 36 ? c - 36 : c / 6; }
  int role;        // 0..5 STM column, 6 state
  int base;        // first lane of the group
  unsigned gmask;  // lanes of the group
  __device__ __forceinline__ int comp(int r) const { return role < 6 ? 6 * r + role : 36 + r; }
  template <typename T>
  __device__ __forceinline__ T from_state(T v) const { return __shfl_sync(gmask, v, base + 6); }
  __device__ __forceinline__ double from(double v, int r) const { return __shfl_sync(gmask, v, base + r); }

  __device__ __forceinline__ void rhs(const double (&v)[6], double mu, const Dir& dir, double (&dv)[6]) const {
    const double x = from_state(v[0]);
    const double y = from_state(v[1]);
    const double z = from_state(v[2]);
    const double vx = from_state(v[3]);
    const double vy = from_state(v[4]);
    const Hess H = hessian_split(*this, role == 6 ? 0 : role, x, y, z, vx, vy, mu);
    if (role < 6) {
      // rows of F(x) @ Phi[:, j] (dynamics/rtbp.py:204-209), zero terms skipped
      dv[0] = v[3];
      dv[1] = v[4];
      dv[2] = v[5];
      dv[3] = ((H.xx * v[0] + H.xy * v[1]) + H.xz * v[2]) + 2.0 * v[4];
      dv[4] = ((H.xy * v[0] + H.yy * v[1]) + H.yz * v[2]) + (-2.0) * v[3];
      dv[5] = (H.xz * v[0] + H.yz * v[1]) + H.zz * v[2];
    } else {
      dv[0] = v[3];
      dv[1] = v[4];
      dv[2] = v[5];
      dv[3] = H.ax;
      dv[4] = H.ay;
      dv[5] = H.az;
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      const int c = comp(r);
      dv[r] = neg_if(dv[r], c >= dir.neg_lo && c < dir.neg_hi);
    }
  }
};

// G = 14 (42-dim state + STM, latency layout): fourteen lanes own one
// trajectory, two per STM column and two for the state; lane 2c + h holds
// rows 3h..3h+2 of column c (components 6(3h + r) + c), lanes 12/13 the
// position / velocity of the state.  The right-hand side: each lane reads its
// partner's three components (lane ^ 1); position lanes' derivatives are
// those components, velocity lanes form rows 3..5 of F(x) Phi[:, c] from
// them and their own, the state's velocity lane takes the accelerations.  The
// Hessian is shared as in G = 7 (jobs 0..5 on lanes 0..5).  Same operations
// and operands as Layout<7>: same bits, at half the stage work per lane.
template <>
struct Layout<14> {
  static constexpr int D = 42;
  static constexpr int NC = 3;
  static constexpr int TPW = 2;
  int role;        // 2c + h (c < 6 STM column, c = 6 state; h = 0 rows 0..2, 1 rows 3..5)
  int base;
  unsigned gmask;
  __device__ __forceinline__ int comp(int r) const {
    const int c = role >> 1, h = role & 1;
    return c < 6 ? 6 * (3 * h + r) + c : 36 + 3 * h + r;
  }
  __device__ __forceinline__ int owner(int c) const { return c >= 36 ? (c < 39 ? 12 : 13) : 2 * (c % 6) + (c / 6 >= 3); }
  __device__ __forceinline__ int local(int c) const { return c >= 36 ? (c - 36) % 3 : (c / 6) % 3; }
  __device__ __forceinline__ double from(double v, int r) const { return __shfl_sync(gmask, v, base + r); }
  __device__ __forceinline__ void rhs(const double (&v)[3], double mu, const Dir& dir, double (&dv)[3]) const {
    const double x = from(v[0], 12), y = from(v[1], 12), z = from(v[2], 12);
    const double vx = from(v[0], 13), vy = from(v[1], 13);
    const Hess H = hessian_split(*this, role < 6 ? role : 0, x, y, z, vx, vy, mu);
    const int partner = role ^ 1;
    const double q0 = from(v[0], partner), q1 = from(v[1], partner), q2 = from(v[2], partner);
    // rows 3..5 of F(x) Phi[:, c] (dynamics/rtbp.py:204-209): q = rows 0..2, v = rows 3..5
    const double r3 = ((H.xx * q0 + H.xy * q1) + H.xz * q2) + 2.0 * v[1];
    const double r4 = ((H.xy * q0 + H.yy * q1) + H.yz * q2) + (-2.0) * v[0];
    const double r5 = (H.xz * q0 + H.yz * q1) + H.zz * q2;
    const bool pos = (role & 1) == 0, state = role >= 12;
    double d0 = pos ? q0 : (state ? H.ax : r3);
    double d1 = pos ? q1 : (state ? H.ay : r4);
    double d2 = pos ? q2 : (state ? H.az : r5);
    dv[0] = neg_if(d0, comp(0) >= dir.neg_lo && comp(0) < dir.neg_hi);
    dv[1] = neg_if(d1, comp(1) >= dir.neg_lo && comp(1) < dir.neg_hi);
    dv[2] = neg_if(d2, comp(2) >= dir.neg_lo && comp(2) < dir.neg_hi);
  }
};

// G = 2 (6-dim state, latency layout): a lane pair owns one trajectory;
// role 0 holds the position (x, y, z), role 1 the velocity.  The right-hand
// side splits by primary: role 0 evaluates the terms of the first primary,
// role 1 those of the second, with one instruction stream and per-lane
// constants; the pair exchanges quotients and then splits the accelerations
// the same way (role 0 forms ax, role 1 ay).  Every operation
// is the one rhs6 performs (x - (1-mu) == x + (-(1-mu)), x - 1 == x + (-1)),
// so the result is bit-identical; the per-step FP64 critical path is about
// half that of G = 1, at ~7% more total work.
template <>
struct Layout<2> {
  static constexpr int D = 6;
  static constexpr int NC = 3;
  static constexpr int TPW = 16;
  int role;        // 0 position, 1 velocity
  int base;        // first lane of the pair
  unsigned gmask;  // the pair
  __device__ __forceinline__ int comp(int r) const { return 3 * role + r; }
  __device__ __forceinline__ int owner(int c) const { return c / 3; }
  __device__ __forceinline__ int local(int c) const { return c % 3; }
  __device__ __forceinline__ void rhs(const double (&v)[3], double mu, const Dir& dir, double (&dv)[3]) const {
    const bool r0 = role == 0;
    const double o0 = __shfl_xor_sync(gmask, v[0], 1);
    const double o1 = __shfl_xor_sync(gmask, v[1], 1);
    const double o2 = __shfl_xor_sync(gmask, v[2], 1);
    const double x = r0 ? v[0] : o0, y = r0 ? v[1] : o1, z = r0 ? v[2] : o2;
    const double vx = r0 ? o0 : v[0], vy = r0 ? o1 : v[1], vz = r0 ? o2 : v[2];
    const double omu = 1.0 - mu;
    const double cb = r0 ? mu : -omu;   // x + cb = x + mu | x - (1 - mu)
    const double a1 = r0 ? mu : -1.0;   // numerator of the x-term: (x + a1) + a2
    const double a2 = r0 ? 0.0 : mu;
    const double mb = r0 ? omu : mu;
    const double mz = r0 ? -omu : mu;
    const double t = x + cb;
    // y*y on role 0 and z*z on role 1 in one multiply, exchanged
    const double w = r0 ? y : z;
    const double sq = w * w;
    const double sqo = __shfl_xor_sync(gmask, sq, 1);
    const double yy = r0 ? sq : sqo;
    const double zz = r0 ? sqo : sq;
    const double r = sqrt((t * t + yy) + zz);
    const double rc = r * (r * r);
    const double ir = hg_rcp_rn(rc);
    const double qx = hg_div_rn(mb * ((x + a1) + a2), rc, ir);
    const double qy = hg_div_rn(mb * y, rc, ir);
    const double qz = hg_div_rn(mz * z, rc, ir);
    // The accelerations ((2 vy + x) - q1x) - q2x and ((-2 vx + y) - q1y) - q2y
    // (q1 the first primary's quotient, role 0's; q2 the second's, role 1's)
    // in one instruction stream: role 0 forms ax, role 1 ay, and role 1
    // takes ax from its partner; az = q1z - q2z on role 1.
    const double p = __shfl_xor_sync(gmask, r0 ? qy : qx, 1);  // role 0: the second qx; role 1: the first qy
    const double pz = __shfl_xor_sync(gmask, qz, 1);
    const double q1 = r0 ? qx : p;
    const double q2 = r0 ? p : qy;
    const double acc = (((r0 ? 2.0 : -2.0) * (r0 ? vy : vx) + (r0 ? x : y)) - q1) - q2;
    const double ax = __shfl_xor_sync(gmask, acc, 1);
    const double az = pz - qz;
    dv[0] = r0 ? vx : ax;
    dv[1] = r0 ? vy : acc;
    dv[2] = r0 ? vz : az;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int c = comp(i);
      dv[i] = neg_if(dv[i], c >= dir.neg_lo && c < dir.neg_hi);
    }
  }
};

// G = 6 (6-dim state, lowest-latency layout): six lanes own one trajectory,
// lane `role` holds component `role`, five trajectories per warp (lanes 30
// and 31 idle).  The right-hand side splits the six quotients of rhs6 over
// the six lanes: lane (b, a) with b = role / 3 the primary and a = role % 3
// the axis forms the numerator of axis a over r_b^3 (each primary's lanes
// compute its distance redundantly, in parallel); the acceleration lanes
// 3..5 fetch the first primary's quotient of their axis and combine.  Every
// operation and its operands are the ones rhs6 uses, so the bits are too;
// the per-step FP64 critical path is about 0.55x that of G = 2.
template <>
struct Layout<6> {
  static constexpr int D = 6;
  static constexpr int NC = 1;
  static constexpr int TPW = 5;
  int role;        // component 0..5
  int base;        // first lane of the group
  unsigned gmask;  // the six lanes
  __device__ __forceinline__ int comp(int) const { return role; }
  __device__ __forceinline__ int owner(int c) const { return c; }
  __device__ __forceinline__ int local(int) const { return 0; }
  __device__ __forceinline__ void rhs(const double (&v)[1], double mu, const Dir& dir, double (&dv)[1]) const {
    const double x = __shfl_sync(gmask, v[0], base);
    const double y = __shfl_sync(gmask, v[0], base + 1);
    const double z = __shfl_sync(gmask, v[0], base + 2);
    // lanes 0..2: their derivative is the velocity of lane role + 3; lanes
    // 3 and 4: the Coriolis term needs vy (lane 4) and vx (lane 3)
    const int src = role < 3 ? role + 3 : (role == 3 ? 4 : 3);
    const double u = __shfl_sync(gmask, v[0], base + src);
    const bool b0 = role < 3;
    const int ax = b0 ? role : role - 3;
    const double omu = 1.0 - mu;
    const double cb = b0 ? mu : -omu;  // x + mu | x - (1 - mu)
    const double a1 = b0 ? mu : -1.0;  // x-numerator: (x + a1) + a2
    const double a2 = b0 ? 0.0 : mu;
    const double t = x + cb;
    // the squares t_b^2, y^2, z^2 in one multiply: lane (b, a) squares t_b,
    // y or z for a = 0, 1, 2, and each lane gathers its primary's three
    const double w = ax == 0 ? t : (ax == 1 ? y : z);
    const double sq = w * w;
    const double tt = __shfl_sync(gmask, sq, base + (b0 ? 0 : 3));
    const double yy = __shfl_sync(gmask, sq, base + 1);
    const double zz = __shfl_sync(gmask, sq, base + 2);
    const double r = sqrt((tt + yy) + zz);
    const double rc = r * (r * r);
    const double ir = hg_rcp_rn(rc);
    const double nx = (x + a1) + a2;
    const double nb = ax == 0 ? nx : (ax == 1 ? y : z);
    const double m = b0 ? (ax == 2 ? -omu : omu) : mu;
    const double q = hg_div_rn(m * nb, rc, ir);
    // first primary's quotient of this lane's axis (lanes 3..5 use it)
    const double pq = __shfl_sync(gmask, q, base + ax);
    const double c2 = role == 3 ? 2.0 : -2.0;
    const double xy = role == 3 ? x : y;
    const double acc_xy = ((c2 * u + xy) - pq) - q;
    const double acc_z = pq - q;
    const double d = role < 3 ? u : (role == 5 ? acc_z : acc_xy);
    dv[0] = neg_if(d, role >= dir.neg_lo && role < dir.neg_hi);
  }
};

// numpy float64 dot order of the host the reference fixtures come from:
// sequential fused accumulation for n < 16, a 32-element blocked sum plus a
// fused tail for n = 42.  v is the full vector (identical in every lane).
// This single-lane statement defines the order; the kernels evaluate it
// spread over a lane group (dots42_group, and the Gather<G> helpers below).
template <int D>
__device__ __forceinline__ double np_dot_self(const double* v) {
  if constexpr (D == 6) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) s = fma(v[i], v[i], s);
    return s;
  } else {
    double a[4][4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int m = 0; m < 4; ++m) a[k][m] = v[8 * k + m] * v[8 * k + m] + v[8 * k + 4 + m] * v[8 * k + 4 + m];
    double s[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) s[m] = ((a[0][m] + a[1][m]) + a[2][m]) + a[3][m];
    double dot = (s[0] + s[2]) + (s[1] + s[3]);
#pragma unroll
    for (int i = 32; i < 42; ++i) dot = fma(v[i], v[i], dot);
    return dot;
  }
}

// Both np_dot_self<42> of the 42-vectors va and vb (shared memory) over a
// lane group of at least six lanes (L.role, L.base, L.gmask; role r acts as
// r % 6).  The sixteen blocked terms a[k][m] = v[8k+m]^2 + v[8k+4+m]^2 of
// each vector are spread over three lanes (va on roles 0..2, vb on 3..5),
// gathered by shuffle, and the two reductions (blocked sums, then the fused
// tail over components 32..41) run side by side on the two halves: the same
// operations in the same order as np_dot_self<42>, ~43 FP64 instructions per
// lane for both norms instead of ~146.
template <class LT>
__device__ __forceinline__ void dots42_group(const LT& L, const double* va, const double* vb, double& da, double& db) {
  const int r = L.role % 6;
  const bool second = r >= 3;
  const double* v = second ? vb : va;
  const int r3 = second ? r - 3 : r;
  const int off = second ? 3 : 0;
  double aj[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int j = r3 + 3 * i;
    const int jj = j < 16 ? j : 15;
    const int b0 = 8 * (jj >> 2) + (jj & 3);
    aj[i] = v[b0] * v[b0] + v[b0 + 4] * v[b0 + 4];
  }
  double a[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) a[j] = __shfl_sync(L.gmask, aj[j / 3], L.base + off + j % 3);
  double sm[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) sm[m] = ((a[m] + a[4 + m]) + a[8 + m]) + a[12 + m];
  double dot = (sm[0] + sm[2]) + (sm[1] + sm[3]);
#pragma unroll
  for (int i = 32; i < 42; ++i) dot = fma(v[i], v[i], dot);
  da = __shfl_sync(L.gmask, dot, L.base);
  db = __shfl_sync(L.gmask, dot, L.base + 3);
}

// Squared 2-norm of the full D-vector whose 6 components per lane are v, in
// the numpy dot order above.  G = 1: the vector is the lane's own registers;
// G = 7: the group assembles it in a 42-double shared-memory slot.
template <int G>
struct Gather;
template <>
struct Gather<1> {
  __device__ __forceinline__ double dot(const Layout<1>&, const double (&v)[6]) const {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) s = fma(v[i], v[i], s);
    return s;
  }
  __device__ __forceinline__ void dot2(const Layout<1>& L, const double (&a)[6], const double (&b)[6], double& da,
                                       double& db) const {
    da = dot(L, a);
    db = dot(L, b);
  }
};
template <>
struct Gather<7> {
  double* slot;  // 84 doubles in shared memory (two 42-vectors)
  __device__ __forceinline__ void dot2(const Layout<7>& L, const double (&a)[6], const double (&b)[6], double& da,
                                       double& db) const {
    __syncwarp(L.gmask);
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      slot[L.comp(r)] = a[r];
      slot[42 + L.comp(r)] = b[r];
    }
    __syncwarp(L.gmask);
    dots42_group(L, slot, slot + 42, da, db);
  }
};

template <>
struct Gather<14> {
  double* slot;  // 84 doubles in shared memory (two 42-vectors)
  __device__ __forceinline__ void dot2(const Layout<14>& L, const double (&a)[3], const double (&b)[3], double& da,
                                       double& db) const {
    __syncwarp(L.gmask);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      slot[L.comp(r)] = a[r];
      slot[42 + L.comp(r)] = b[r];
    }
    __syncwarp(L.gmask);
    dots42_group(L, slot, slot + 42, da, db);
  }
};

template <>
struct Gather<2> {
  // sequential fused accumulation over components 0..5: the position lane's
  // partial sum seeds the velocity lane's
  __device__ __forceinline__ double dot(const Layout<2>& L, const double (&v)[3]) const {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) s = fma(v[i], v[i], s);
    s = __shfl_sync(L.gmask, s, L.base);
#pragma unroll
    for (int i = 0; i < 3; ++i) s = fma(v[i], v[i], s);
    return __shfl_sync(L.gmask, s, L.base + 1);
  }
  // the two dots side by side, each the same sequential fused accumulation
  // over components 0..5: role 0 accumulates a, role 1 b; one exchange per
  // component gives role 0 the partner's a (components 3..5) and role 1 the
  // partner's b (components 0..2)
  __device__ __forceinline__ void dot2(const Layout<2>& L, const double (&a)[3], const double (&b)[3], double& da,
                                       double& db) const {
    const bool r0 = L.role == 0;
    double u[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) u[i] = __shfl_xor_sync(L.gmask, r0 ? b[i] : a[i], 1);
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double c = r0 ? a[i] : u[i];
      s = fma(c, c, s);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double c = r0 ? u[i] : b[i];
      s = fma(c, c, s);
    }
    da = __shfl_sync(L.gmask, s, L.base);
    db = __shfl_sync(L.gmask, s, L.base + 1);
  }
};

template <>
struct Gather<6> {
  // every lane runs the sequential fused accumulation over the six
  // broadcast components
  __device__ __forceinline__ double dot(const Layout<6>& L, const double (&v)[1]) const {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const double c = __shfl_sync(L.gmask, v[0], L.base + i);
      s = fma(c, c, s);
    }
    return s;
  }
  // the two dots in the same six fused multiply-adds: lanes 0..2 accumulate
  // a, lanes 3..5 b, then each is broadcast
  __device__ __forceinline__ void dot2(const Layout<6>& L, const double (&a)[1], const double (&b)[1], double& da,
                                       double& db) const {
    const bool first = L.role < 3;
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const double ca = __shfl_sync(L.gmask, a[0], L.base + i);
      const double cb = __shfl_sync(L.gmask, b[0], L.base + i);
      const double c = first ? ca : cb;
      s = fma(c, c, s);
    }
    da = __shfl_sync(L.gmask, s, L.base);
    db = __shfl_sync(L.gmask, s, L.base + 3);
  }
};

// v[r] for a runtime r without dynamic register indexing.
template <int NC>
__device__ __forceinline__ double pick(const double (&v)[NC], int r) {
  double o = v[0];
#pragma unroll
  for (int i = 1; i < NC; ++i) o = (r == i) ? v[i] : o;
  return o;
}

// ---------------------------------------------------------------------------
// Step-size helpers, integrators/utils.py:126-296
// ---------------------------------------------------------------------------
// The step bounds are > 0 and not NaN (the entry points check them), so the
// comparisons with them run on the integer pipes.
__device__ __forceinline__ double clamp_step(double h, double max_step, double min_step) {
  if (hg_gt_pos(h, hg_bits(max_step))) h = max_step;
  if (hg_lt_pos(h, hg_bits(min_step))) h = min_step;
  return h;
}
__device__ __forceinline__ double adjust_step_to_endpoint(double t, double h, double t_end) {
  if (hg_gt(t + h, t_end)) return fabs(t_end - t);
  return h;
}
__device__ __forceinline__ double select_initial_step(double d0, double d1, double min_step, double max_step) {
  double h;
  if (d0 < 1.0e-5 || d1 < 1.0e-5)
    h = 1.0e-6;
  else
    h = (0.01 * d0) / d1;
  if (h > max_step) h = max_step;
  if (h < min_step) h = min_step;
  return h;
}
// exp(e * (Lh + Ll)) rounded once: the composition hg_pow uses after its
// logarithm (two_prod of the exponent with the double-double log).
__device__ __forceinline__ double exp_scaled(double e, double Lh, double Ll) {
  double th, pe, Th, Tl;
  hg_two_prod(e, Lh, th, pe);
  hg_fast_two_sum(th, fma(e, Ll, pe), Th, Tl);
  return hg_exp_dd(Th, Tl);
}

// PI step-size factor after an attempted step (integrators/utils.py
// step-size control, order 8): an accepted step scales h by
// 0.9 * err^-beta * err_prev^alpha (beta = 1/9, alpha = 0.4 beta;
// err_prev^alpha was computed at the previous accepted step and is carried
// in prev_pow), a rejected one by 0.9 * err^(-1/8); factors are clamped to
// [0.2, 10].  Accepting and rejecting lanes share the logarithm, so a warp
// whose trajectories disagree runs one transcendental sequence, not two; in
// a group of lanes the two exponentials run on two lanes at once.  Every
// power is the correctly rounded one hg_pow gives.  Zero, NaN and
// err >= 1e300 take no logarithm: their factors are the clamp bounds (a
// rejected err >= 1e300 gives 0.9 * err^(-1/8) < 0.2).
template <class LT>
__device__ __forceinline__ double pi_factor(const LT& L, bool accepted, double err, double err_prev,
                                            double& prev_pow) {
  const double beta = 1.0 / (8.0 + 1.0);
  const double alpha = 0.4 * beta;
  const double rexp = 1.0 / 8.0;
  const bool regular = hg_in_open_pos(err, HG_BITS_1E300);  // 0 < err < 1e300
  double p1 = 0.0, pa = 0.0;
  if (regular) {
    double Lh, Ll;
    hg_log_dd(err, Lh, Ll);
    const double e1 = accepted ? -beta : -rexp;
    if constexpr (std::is_same_v<LT, Layout<1>>) {
      p1 = exp_scaled(e1, Lh, Ll);
      pa = exp_scaled(alpha, Lh, Ll);
    } else {
      const double v = exp_scaled(L.role == 0 ? e1 : alpha, Lh, Ll);
      p1 = __shfl_sync(L.gmask, v, L.base);
      pa = __shfl_sync(L.gmask, v, L.base + 1);
    }
  }
  double factor;
  if (accepted) {
    if (hg_eq0(err)) {
      factor = 10.0;
      prev_pow = 0.0;
    } else {
      factor = hg_lt0(err_prev) ? 0.9 * p1 : (0.9 * p1) * prev_pow;
      prev_pow = pa;
      if (hg_isnan_cmp(factor)) factor = 10.0;
    }
  } else {
    factor = regular ? 0.9 * p1 : 0.2;
    if (hg_isnan_cmp(factor)) factor = 0.2;
  }
  if (hg_lt_pos(factor, HG_BITS_0_2)) factor = 0.2;
  if (hg_gt_pos(factor, HG_BITS_10)) factor = 10.0;
  return factor;
}

// integrators/utils.py:13-68
// (the sign tests on the integer pipes: hg_lt0 / hg_gt0 / hg_eq0 equal
// g < 0, g > 0, g == 0)
__device__ __forceinline__ bool event_crossed(double g_prev, double g_new, int dir) {
  if (dir == 0) return (hg_lt0(g_prev) && hg_gt0(g_new)) || (hg_gt0(g_prev) && hg_lt0(g_new)) || hg_eq0(g_new);
  if (dir > 0) return (hg_lt0(g_prev) && hg_gt0(g_new)) || hg_eq0(g_new);
  return (hg_gt0(g_prev) && hg_lt0(g_new)) || hg_eq0(g_new);
}
__device__ __forceinline__ bool crossed_direction(double g_left, double g_mid, int dir) {
  if (dir == 0) return (g_left < 0.0 && g_mid > 0.0) || (g_left > 0.0 && g_mid < 0.0);
  if (dir > 0) return (g_left < 0.0 && g_mid > 0.0);
  return (g_left > 0.0 && g_mid < 0.0);
}

// numpy.maximum(|a|, |b|) on the integer pipe: the bit patterns of
// non-negative doubles order like unsigned integers, and a NaN pattern
// compares above +inf, so NaN propagates as numpy's maximum does.
__device__ __forceinline__ double np_maximum_abs(double a, double b) {
  const unsigned long long ua = (unsigned long long)__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long ub = (unsigned long long)__double_as_longlong(b) & 0x7FFFFFFFFFFFFFFFull;
  return __longlong_as_double((long long)(ua > ub ? ua : ub));
}

// isfinite on the integer pipe (exponent field not all ones).
__device__ __forceinline__ bool finite_bits(double a) {
  return ((unsigned long long)__double_as_longlong(a) & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}

// ---------------------------------------------------------------------------
// Fixed-step RK kernels, integrators/rk.py:154-215 and :531-588
// ---------------------------------------------------------------------------
// The products h * a_ij and h * b_j of one fixed step, formed where they
// are used (every lane of a trajectory forms all of them).
template <int ORDER>
struct InlineCoef {
  double h;
  template <int I, int J>
  __device__ __forceinline__ double a() const {
    return h * FixedTab<ORDER>::a(I, J);
  }
  template <int J>
  __device__ __forceinline__ double b() const {
    return h * FixedTab<ORDER>::b(J);
  }
};

// Position of a_ij (i >= 1, j < i, nonzero) in the list of the tableau's
// nonzero A entries by rows, followed by the nonzero B entries (b_j at
// fixed_flat(S, j)); -1 for a zero entry.
template <int ORDER>
__host__ __device__ constexpr int fixed_flat(int i, int j) {
  using T = FixedTab<ORDER>;
  int q = 0;
  for (int r = 1; r < T::S; ++r)
    for (int c = 0; c < r; ++c) {
      if (T::a(r, c) != 0.0) {
        if (r == i && c == j) return q;
        ++q;
      }
    }
  for (int c = 0; c < T::S; ++c) {
    if (T::b(c) != 0.0) {
      if (i == T::S && c == j) return q;
      ++q;
    }
  }
  return -1;
}

// The same products spread over a warp whose lanes all step with the same h
// (fixed-step runs): lane l forms the products of list positions l, l + 32
// and l + 64 (three FP64 multiplies per step instead of one per entry) and
// each stage fetches its coefficients by shuffle.  Bit-identical: every
// product is the same h * a.  All 32 lanes must be present.
template <int ORDER>
struct WarpCoef {
  static_assert(fixed_flat<ORDER>(FixedTab<ORDER>::S, FixedTab<ORDER>::S) < 0, "");
  double base[3];  // this lane's tableau entries
  double v[3];     // this lane's products for the current step
  __device__ __forceinline__ explicit WarpCoef(int lane) {
    using T = FixedTab<ORDER>;
    base[0] = base[1] = base[2] = 0.0;
    static_for<T::S>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      static_for<i>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        if constexpr (T::a(i, j) != 0.0) {
          constexpr int q = fixed_flat<ORDER>(i, j);
          static_assert(q >= 0 && q < 96, "");
          if (lane == q % 32) base[q / 32] = T::a(i, j);
        }
      });
    });
    static_for<T::S>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      if constexpr (T::b(j) != 0.0) {
        constexpr int q = fixed_flat<ORDER>(T::S, j);
        static_assert(q >= 0 && q < 96, "");
        if (lane == q % 32) base[q / 32] = T::b(j);
      }
    });
  }
  __device__ __forceinline__ void set_step(double h) {
    v[0] = h * base[0];
    v[1] = h * base[1];
    v[2] = h * base[2];
  }
  template <int I, int J>
  __device__ __forceinline__ double a() const {
    constexpr int q = fixed_flat<ORDER>(I, J);
    return __shfl_sync(0xFFFFFFFFu, v[q / 32], q % 32);
  }
  template <int J>
  __device__ __forceinline__ double b() const {
    constexpr int q = fixed_flat<ORDER>(FixedTab<ORDER>::S, J);
    return __shfl_sync(0xFFFFFFFFu, v[q / 32], q % 32);
  }
};

template <int ORDER, class LT, class CF>
__device__ __forceinline__ void rk_fixed_step(const LT& L, const double (&y)[LT::NC], const CF& cf, double mu,
                                              const Dir& dir, double (&yn)[LT::NC]) {
  using T = FixedTab<ORDER>;
  constexpr int NC = LT::NC;
  double k[T::S][NC];
  L.rhs(y, mu, dir, k[0]);
  static_for<T::S - 1>([&](auto ic) {
    constexpr int i = decltype(ic)::value + 1;
    double ys[NC];
#pragma unroll
    for (int d = 0; d < NC; ++d) ys[d] = y[d];
    static_for<i>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      if constexpr (T::a(i, j) != 0.0) {
        const double c = cf.template a<i, j>();
#pragma unroll
        for (int d = 0; d < NC; ++d) ys[d] = ys[d] + c * k[j][d];
      }
    });
    L.rhs(ys, mu, dir, k[i]);
  });
#pragma unroll
  for (int d = 0; d < NC; ++d) yn[d] = y[d];
  static_for<T::S>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    if constexpr (T::b(j) != 0.0) {
      const double c = cf.template b<j>();
#pragma unroll
      for (int d = 0; d < NC; ++d) yn[d] = yn[d] + c * k[j][d];
    }
  });
}

template <int ORDER, class LT>
__device__ __forceinline__ void rk_fixed_step(const LT& L, const double (&y)[LT::NC], double h, double mu,
                                              const Dir& dir, double (&yn)[LT::NC]) {
  rk_fixed_step<ORDER>(L, y, InlineCoef<ORDER>{h}, mu, dir, yn);
}

struct FixedParams {
  int N;
  double mu;
  Dir dir;
  const double* y0;  // [D][ld_in]
  long long ld_in;
  const double* t_vals;  // [n]
  int n;
  int out_every;      // write rows 0, out_every, 2*out_every, ... (and nothing else)
  double* out;        // [n_out][D][ld_out]
  long long ld_out;
  int* status;        // [N] or null
  // optional terminal plane event g = y[ev_index] - ev_offset (ev_index < 0: none)
  int ev_index;
  double ev_offset;
  int ev_dir;
  double xtol, gtol;
  double* hit_t;  // [ld_out]
  double* hit_y;  // [D][ld_out]
  int* n_hits;    // [N]
};

// _hermite_eval_dense (integrators/rk.py:286-327) for one component.
__device__ __forceinline__ double hermite_eval(double y0, double f0, double y1, double f1, double x, double h) {
  const double x2 = x * x;
  const double x3 = x2 * x;
  const double H00 = (2.0 * x3 - 3.0 * x2) + 1.0;
  const double H10 = (x3 - 2.0 * x2) + x;
  const double H01 = -2.0 * x3 + 3.0 * x2;
  const double H11 = x3 - x2;
  return ((H00 * y0 + H10 * (h * f0)) + H01 * y1) + H11 * (h * f1);
}

// Fixed step with a terminal plane event: integrators/rk.py:655-718
// (_integrate_fixed_rk_until_event) and :330-391 (_hermite_refine_in_step).
// Each step also evaluates f(y_{n+1}) for the cubic Hermite interpolant;
// rows after the crossing are not written (the reference returns
// [y0, y_hit] only).
template <int ORDER, int G>
__global__ void __launch_bounds__(128) fixed_rk_event_kernel(FixedParams p) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  Layout<G> L;
  int traj;
  if constexpr (G == 1) {
    L.role = 6;
    traj = warp * 32 + lane;
  } else {
    if (lane >= 28) return;
    const int g = lane / 7;
    L.role = lane % 7;
    L.base = g * 7;
    L.gmask = 0x7Fu << L.base;
    traj = warp * 4 + g;
  }
  if (traj >= p.N) return;
  const bool leader = (G == 1) || L.role == 6;
  int ev_r = L.local(p.ev_index);
  bool ev_mine = true;
  int ev_src = lane;
  if constexpr (G == 7) {
    ev_mine = (L.role == L.owner(p.ev_index));
    ev_src = L.base + L.owner(p.ev_index);
  }
  auto bcast = [&](double v) -> double {
    if constexpr (G == 1)
      return v;
    else
      return __shfl_sync(L.gmask, v, ev_src);
  };
  double y[6];
#pragma unroll
  for (int r = 0; r < 6; ++r) y[r] = p.y0[(long long)L.comp(r) * p.ld_in + traj];
#pragma unroll
  for (int r = 0; r < 6; ++r) p.out[(long long)L.comp(r) * p.ld_out + traj] = y[r];
  const long long row = (long long)Layout<G>::D * p.ld_out;
  double f_prev[6];
  L.rhs(y, p.mu, p.dir, f_prev);
  double g_prev = bcast(ev_mine ? (pick<6>(y, ev_r) - p.ev_offset) : 0.0);
  bool finite = true;
  int hit = 0;
  for (int idx = 0; idx < p.n - 1; ++idx) {
    const double t_n = p.t_vals[idx];
    const double h = p.t_vals[idx + 1] - t_n;
    double yn[6], f_new[6];
    rk_fixed_step<ORDER>(L, y, h, p.mu, p.dir, yn);
    L.rhs(yn, p.mu, p.dir, f_new);
    const double g_new = bcast(ev_mine ? (pick<6>(yn, ev_r) - p.ev_offset) : 0.0);
    if (event_crossed(g_prev, g_new, p.ev_dir)) {
      const double ye = pick<6>(y, ev_r), fe0 = pick<6>(f_prev, ev_r), ye1 = pick<6>(yn, ev_r),
                   fe1 = pick<6>(f_new, ev_r);
      double a = 0.0, b = 1.0, g_left = g_prev, x_hit = -1.0;
      for (int it = 0; it < 128; ++it) {
        const double mid = 0.5 * (a + b);
        const double g_mid = bcast(ev_mine ? (hermite_eval(ye, fe0, ye1, fe1, mid, h) - p.ev_offset) : 0.0);
        if (fabs(g_mid) <= p.gtol) {
          x_hit = mid;
          break;
        }
        if (crossed_direction(g_left, g_mid, p.ev_dir)) {
          b = mid;
        } else {
          a = mid;
          g_left = g_mid;
        }
        if ((b - a) * fabs(h) <= p.xtol) break;
      }
      if (x_hit < 0.0) x_hit = b;
      if (leader) p.hit_t[traj] = t_n + x_hit * h;
#pragma unroll
      for (int r = 0; r < 6; ++r)
        p.hit_y[(long long)L.comp(r) * p.ld_out + traj] = hermite_eval(y[r], f_prev[r], yn[r], f_new[r], x_hit, h);
      hit = 1;
      break;
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      y[r] = yn[r];
      f_prev[r] = f_new[r];
      finite = finite && finite_bits(yn[r]);
    }
    g_prev = g_new;
    if ((idx + 1) % p.out_every == 0) {
      double* o = p.out + (long long)((idx + 1) / p.out_every) * row;
#pragma unroll
      for (int r = 0; r < 6; ++r) o[(long long)L.comp(r) * p.ld_out + traj] = y[r];
    }
  }
  if constexpr (G == 7) finite = __all_sync(L.gmask, finite);
  if (leader) {
    p.n_hits[traj] = hit;
    if (p.status) p.status[traj] = finite ? HG_OK : HG_NONFINITE;
  }
}

template <int ORDER, int G>
__global__ void __launch_bounds__(128) fixed_rk_kernel(FixedParams p) {
  constexpr int NC = Layout<G>::NC;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  Layout<G> L;
  int traj;
  if constexpr (G == 1) {
    L.role = 6;
    traj = warp * 32 + lane;
  } else if constexpr (G == 14) {
    if (lane >= 28) return;
    const int g = lane / 14;
    L.role = lane % 14;
    L.base = g * 14;
    L.gmask = 0x3FFFu << L.base;
    traj = warp * 2 + g;
  } else {
    if (lane >= 28) return;
    const int g = lane / 7;
    L.role = lane % 7;
    L.base = g * 7;
    L.gmask = 0x7Fu << L.base;
    traj = warp * 4 + g;
  }
  if (traj >= p.N) return;
  double y[NC];
#pragma unroll
  for (int r = 0; r < NC; ++r) y[r] = p.y0[(long long)L.comp(r) * p.ld_in + traj];
#pragma unroll
  for (int r = 0; r < NC; ++r) p.out[(long long)L.comp(r) * p.ld_out + traj] = y[r];
  const long long row = (long long)Layout<G>::D * p.ld_out;
  bool finite = true;
  for (int idx = 0; idx < p.n - 1; ++idx) {
    const double h = p.t_vals[idx + 1] - p.t_vals[idx];
    double yn[NC];
    rk_fixed_step<ORDER>(L, y, h, p.mu, p.dir, yn);
#pragma unroll
    for (int r = 0; r < NC; ++r) {
      y[r] = yn[r];
      finite = finite && finite_bits(yn[r]);
    }
    if ((idx + 1) % p.out_every == 0) {
      double* o = p.out + (long long)((idx + 1) / p.out_every) * row;
#pragma unroll
      for (int r = 0; r < NC; ++r) o[(long long)L.comp(r) * p.ld_out + traj] = y[r];
    }
  }
  if (p.status) {
    if constexpr (G > 1) {
      finite = __all_sync(L.gmask, finite);
      // one lane of the group writes the status
      if (L.role != (G == 7 ? 6 : 0)) return;
    }
    p.status[traj] = finite ? HG_OK : HG_NONFINITE;
  }
}

// ---------------------------------------------------------------------------
// DOP853, integrators/rk.py:1636-1708, :1790-2102, :2375-2549, :2678-2803
// ---------------------------------------------------------------------------
struct DopParams {
  int N;
  double mu;
  Dir dir;
  const double* y0;  // [D][ld]
  long long ld;
  const double* t0_arr;  // [N] or null -> t0
  const double* tmax_arr;
  double t0, tmax;
  double rtol, atol, max_step, min_step;
  long long max_steps;
  // plane event g = y[ev_index] - ev_offset (ev_index < 0: none)
  int ev_index;
  double ev_offset;
  int ev_dir;
  int max_hits;
  double xtol, gtol;
  // dense samples at linspace(t0_i, tmax_i, m) (m >= 2); dense_last: only the
  // final sample is evaluated and written (row 0 of y_out)
  int m;
  int dense_last;
  double* y_out;  // [m or 1][D][ld]
  // outputs
  double* y_end;  // [D][ld]
  double* t_end;  // [N]
  double* hit_t;  // [max_hits][ld]
  double* hit_y;  // [max_hits][D][ld]
  int* n_hits;
  int* n_accept;
  int* n_reject;
  int* status;
  // persistent lane refill
  int* next_traj;  // scratch counter (zeroed before launch) or null: static assignment
  int stride;      // trajectories assigned in the first wave (grid lanes / G)
  // Segmented execution (seg != 0): the launch advances the trajectories
  // listed in active_in[0 .. *n_in) by at most seg_steps attempted steps.
  // The integration state persists between launches in the outputs (y_end,
  // t_end, n_accept, n_reject, n_hits, status = HG_RUNNING) and in ws_*;
  // unfinished trajectories are appended to active_out (count *n_out).
  // Each launch starts every group with a full set of live trajectories, so
  // lanes that finished early stop wasting the FP64 pipe.
  int seg;
  int seg_steps;
  const int* active_in;
  const int* n_in;
  int* active_out;
  int* n_out;
  double* ws_h;
  double* ws_err_prev;
  double* ws_prev_pow;
  int* ws_q;
  // Deferred refinement of event crossings (rec != null): every crossing step
  // is appended to a record pool (save_step: record slot, its trajectory in
  // refine_list and hit index in refine_hit) and refine_kernel computes
  // hit_t / hit_y for records [0 .. *refine_count), all lanes in lock step.
  // Capacity rec_ld >= N * max_hits (no trajectory records more hits).
  double* rec;
  long long rec_ld;
  int* refine_list;
  int* refine_hit;
  int* refine_count;
};

#define HG_RUNNING (-1)

// Position of the nonzero a_ij (1 <= i < 12, j < i) in DOP853's list of
// nonzero stage coefficients by rows, followed by the nonzero b_j
// (dop_flat(12, j)); -1 for a zero entry.  dop_nnz(): the list's length.
__host__ __device__ constexpr int dop_flat(int i, int j) {
  int q = 0;
  for (int r = 1; r < DopTab::S; ++r)
    for (int c = 0; c < r; ++c) {
      if (DopTab::a(r, c) != 0.0) {
        if (r == i && c == j) return q;
        ++q;
      }
    }
  for (int c = 0; c < DopTab::S; ++c) {
    if (DopTab::b(c) != 0.0) {
      if (i == DopTab::S && c == j) return q;
      ++q;
    }
  }
  return -1;
}
__host__ __device__ constexpr int dop_first_nonzero_e(bool e5) {
  for (int j = 0; j < 13; ++j)
    if ((e5 ? DopTab::e5(j) : DopTab::e3(j)) != 0.0) return j;
  return -1;
}
__host__ __device__ constexpr int dop_nnz() {
  int q = 0;
  for (int r = 1; r < DopTab::S; ++r)
    for (int c = 0; c < r; ++c) q += DopTab::a(r, c) != 0.0;
  for (int c = 0; c < DopTab::S; ++c) q += DopTab::b(c) != 0.0;
  return q;
}

// The products h * a_ij, h * b_j of one DOP853 step, formed where they are
// used (one lane per trajectory).
struct DopInlineCoef {
  double h;
  __device__ __forceinline__ void set_step(double hh) { h = hh; }
  template <int I, int J>
  __device__ __forceinline__ double a() const {
    return h * DopTab::a(I, J);
  }
  template <int J>
  __device__ __forceinline__ double b() const {
    return h * DopTab::b(J);
  }
};

// The list of nonzero coefficients itself (a_ij by rows, then b_j), written
// into shared memory by the block's threads (entry q by thread q mod the
// block size) before any lane leaves: `tab` must hold dop_nnz() doubles and
// be followed by __syncthreads().
__device__ __forceinline__ void dop_coef_table_init(double* tab) {
  static_for<DopTab::S>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    static_for<i>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      if constexpr (DopTab::a(i, j) != 0.0) {
        if ((unsigned)dop_flat(i, j) % blockDim.x == threadIdx.x) tab[dop_flat(i, j)] = DopTab::a(i, j);
      }
    });
  });
  static_for<DopTab::S>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    if constexpr (DopTab::b(j) != 0.0) {
      if ((unsigned)dop_flat(DopTab::S, j) % blockDim.x == threadIdx.x) tab[dop_flat(DopTab::S, j)] = DopTab::b(j);
    }
  });
}

// The same products spread over the NL lanes of a trajectory's group (its h
// is group-uniform): lane r forms list positions r, r + NL, ... from the
// shared-memory table (ceil(58 / NL) FP64 multiplies per step instead of 58)
// and the stages fetch them by shuffle within the group.  Bit-identical:
// every product is the same h * a.
template <int NL>
struct DopGroupCoef {
  static constexpr int K = dop_nnz();
  static constexpr int P = (K + NL - 1) / NL;
  const double* tab;  // dop_coef_table_init
  int r;              // this lane's share
  int src;            // first lane of the group
  unsigned gmask;     // the group's lanes
  double v[P];
  __device__ __forceinline__ DopGroupCoef(const double* table, int share, int group_base, unsigned mask)
      : tab(table), r(share), src(group_base), gmask(mask) {}
  __device__ __forceinline__ void set_step(double h) {
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const int q = r + NL * i;
      v[i] = h * (q < K ? tab[q] : 0.0);
    }
  }
  template <int I, int J>
  __device__ __forceinline__ double a() const {
    constexpr int q = dop_flat(I, J);
    static_assert(q >= 0, "");
    return __shfl_sync(gmask, v[q / NL], src + q % NL);
  }
  template <int J>
  __device__ __forceinline__ double b() const {
    constexpr int q = dop_flat(DopTab::S, J);
    static_assert(q >= 0, "");
    return __shfl_sync(gmask, v[q / NL], src + q % NL);
  }
};

// Row I of the step's coefficients (I < 12: the stage row a_Ij; I = 12: the
// solution weights b_j), its count of nonzero entries and the column of the
// k-th of them.
template <int I>
__host__ __device__ constexpr double dop_row_coef(int j) {
  return I < DopTab::S ? DopTab::a(I, j) : DopTab::b(j);
}
template <int I>
__host__ __device__ constexpr int dop_row_nnz() {
  int n = 0;
  for (int j = 0; j < (I < DopTab::S ? I : DopTab::S); ++j) n += dop_row_coef<I>(j) != 0.0;
  return n;
}
template <int I>
__host__ __device__ constexpr int dop_row_col(int k) {
  for (int j = 0; j < (I < DopTab::S ? I : DopTab::S); ++j)
    if (dop_row_coef<I>(j) != 0.0 && k-- == 0) return j;
  return -1;
}

// Lane pairs (G = 2, one step size per pair): the products h * a_ij, h * b_j
// formed row by row at the start of each stage, two per FP64 multiply --
// lane `role` of the pair forms the (2m + role)-th nonzero entry of the row
// -- and exchanged by shuffle: the same products as DopInlineCoef in about
// half the multiplies.  `c` holds the current row's products by column.
struct DopPairCoef {
  double h;
  int role;
  int base;
  unsigned gmask;
  mutable double c[DopTab::S];
  __device__ __forceinline__ void set_step(double hh) { h = hh; }
  template <int I>
  __device__ __forceinline__ void row() const {
    constexpr int n = dop_row_nnz<I>();
    static_for<(n + 1) / 2>([&](auto mc) {
      constexpr int m = decltype(mc)::value;
      constexpr int ja = dop_row_col<I>(2 * m);
      constexpr int jb = 2 * m + 1 < n ? dop_row_col<I>(2 * m + 1) : -1;
      constexpr double aa = dop_row_coef<I>(ja);
      constexpr double ab = jb >= 0 ? dop_row_coef<I>(jb) : aa;
      const double v = h * (role ? ab : aa);
      c[ja] = __shfl_sync(gmask, v, base);
      if constexpr (jb >= 0) c[jb] = __shfl_sync(gmask, v, base + 1);
    });
  }
  template <int I, int J>
  __device__ __forceinline__ double a() const {
    return c[J];
  }
  template <int J>
  __device__ __forceinline__ double b() const {
    return c[J];
  }
};

// Row preparation of a coefficient provider: DopPairCoef forms a row's
// products ahead of its sum; the others form them where they are used.
template <int I, class CF>
__device__ __forceinline__ void dop_coef_row(const CF&) {}
template <int I>
__device__ __forceinline__ void dop_coef_row(const DopPairCoef& cf) {
  cf.template row<I>();
}

template <class LT>
struct DopLaneT {
  static constexpr int NC = LT::NC;
  // one attempted DOP853 step; k[0] = f(t, y) on entry; k[12] = f(t+h, y_high)
  // on exit.
  __device__ __forceinline__ static void step(const LT& L, const double (&y)[NC], double h, double mu,
                                              const Dir& dir, double (&k)[13][NC], double (&yh)[NC],
                                              double (&e5)[NC], double (&e3)[NC]) {
    step(L, y, DopInlineCoef{h}, h, mu, dir, k, yh, e5, e3);
  }
  // the same with the products h * a_ij, h * b_j from `cf` (set for h)
  template <class CF>
  __device__ __forceinline__ static void step(const LT& L, const double (&y)[NC], const CF& cf, double h, double mu,
                                              const Dir& dir, double (&k)[13][NC], double (&yh)[NC],
                                              double (&e5)[NC], double (&e3)[NC]) {
    using T = DopTab;
    static_for<T::S - 1>([&](auto ic) {
      constexpr int i = decltype(ic)::value + 1;
      dop_coef_row<i>(cf);
      double ys[NC];
#pragma unroll
      for (int d = 0; d < NC; ++d) ys[d] = y[d];
      static_for<i>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        if constexpr (T::a(i, j) != 0.0) {
          const double c = cf.template a<i, j>();
#pragma unroll
          for (int d = 0; d < NC; ++d) ys[d] = ys[d] + c * k[j][d];
        }
      });
      L.rhs(ys, mu, dir, k[i]);
    });
    dop_coef_row<T::S>(cf);
#pragma unroll
    for (int d = 0; d < NC; ++d) yh[d] = y[d];
    static_for<T::S>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      if constexpr (T::b(j) != 0.0) {
        const double c = cf.template b<j>();
#pragma unroll
        for (int d = 0; d < NC; ++d) yh[d] = yh[d] + c * k[j][d];
      }
    });
    L.rhs(yh, mu, dir, k[12]);
    // err5 = sum_j E5_j k_j (the reference starts from zeros; the first term
    // is taken as the start here: only the sign of an all-zero sum can
    // differ, and err5 / err3 enter the step control squared)
    static_for<13>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      constexpr double c5 = T::e5(j);
      constexpr double c3 = T::e3(j);
      if constexpr (c5 != 0.0) {
        constexpr bool first = dop_first_nonzero_e(true) == j;
#pragma unroll
        for (int d = 0; d < NC; ++d) e5[d] = first ? c5 * k[j][d] : e5[d] + c5 * k[j][d];
      }
      if constexpr (c3 != 0.0) {
        constexpr bool first = dop_first_nonzero_e(false) == j;
#pragma unroll
        for (int d = 0; d < NC; ++d) e3[d] = first ? c3 * k[j][d] : e3[d] + c3 * k[j][d];
      }
    });
#pragma unroll
    for (int d = 0; d < NC; ++d) {
      e5[d] = e5[d] * h;
      e3[d] = e3[d] * h;
    }
  }

  // _dop853_build_dense_cache: F[0..6][6] for this lane's components.
  __device__ __forceinline__ static void dense_cache(const LT& L, const double (&y_old)[NC],
                                                     const double (&y_new)[NC], double hseg, double mu,
                                                     const Dir& dir, const double (&k)[13][NC],
                                                     double (&F)[7][NC]) {
    using T = DopTab;
    double kx[3][NC];
    static_for<3>([&](auto sc) {
      constexpr int srow = decltype(sc)::value + 13;
      double ys[NC];
#pragma unroll
      for (int d = 0; d < NC; ++d) {
        double acc = 0.0;
        static_for<srow>([&](auto rc) {
          constexpr int r = decltype(rc)::value;
          constexpr double a = T::a(srow, r);
          if constexpr (a != 0.0) {
            if constexpr (r < 13)
              acc = acc + a * k[r][d];
            else
              acc = acc + a * kx[r - 13][d];
          }
        });
        ys[d] = y_old[d] + hseg * acc;
      }
      L.rhs(ys, mu, dir, kx[srow - 13]);
    });
#pragma unroll
    for (int d = 0; d < NC; ++d) {
      const double dy = y_new[d] - y_old[d];
      F[0][d] = dy;
      F[1][d] = hseg * k[0][d] - dy;
      F[2][d] = 2.0 * dy - hseg * (k[12][d] + k[0][d]);
    }
    static_for<4>([&](auto ic) {
      constexpr int irem = decltype(ic)::value;
#pragma unroll
      for (int d = 0; d < NC; ++d) {
        double acc = 0.0;
        static_for<16>([&](auto rc) {
          constexpr int r = decltype(rc)::value;
          constexpr double c = T::d(irem, r);
          if constexpr (c != 0.0) {
            if constexpr (r < 13)
              acc = acc + c * k[r][d];
            else
              acc = acc + c * kx[r - 13][d];
          }
        });
        F[3 + irem][d] = hseg * acc;
      }
    });
  }

  __device__ __forceinline__ static double eval_row(double y_old, const double (&f)[7], double x) {
    double v = 0.0;
#pragma unroll
    for (int i = 6; i >= 0; --i) {
      v = v + f[i];
      if ((6 - i) % 2 == 0)
        v = v * x;
      else
        v = v * (1.0 - x);
    }
    return v + y_old;
  }

  __device__ __forceinline__ static double eval1(double y_old, const double (&F)[7][NC], int d, double x) {
    double v = 0.0;
#pragma unroll
    for (int i = 6; i >= 0; --i) {
      v = v + F[i][d];
      if ((6 - i) % 2 == 0)
        v = v * x;
      else
        v = v * (1.0 - x);
    }
    return v + y_old;
  }
};

template <int G>
using DopLane = DopLaneT<Layout<G>>;

// Step-coefficient provider of a layout: spread over the group for the
// groups of 6 and 14 lanes (few components per lane), formed row by row in
// pairs for lane pairs, formed inline for 1 and 7 (whose lanes have no
// registers to spare).
template <int G>
__host__ __device__ constexpr bool dop_spread_coef() {
  return G == 6 || G == 14;
}
template <int G>
__device__ __forceinline__ auto dop_coef(const Layout<G>& L, const double* tab) {
  if constexpr (dop_spread_coef<G>()) {
    return DopGroupCoef<G>(tab, L.role, L.base, L.gmask);
  } else if constexpr (G == 2) {
    DopPairCoef cf;
    cf.h = 0.0;
    cf.role = L.role;
    cf.base = L.base;
    cf.gmask = L.gmask;
    return cf;
  } else {
    return DopInlineCoef{0.0};
  }
}

// Lane -> (group, role) for one launch; false for the idle lanes of a warp.
template <int G>
__device__ __forceinline__ bool setup_layout(Layout<G>& L, Gather<G>& gat, double* sm_gather, int& traj) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if constexpr (G == 1) {
    L.role = 6;
    traj = warp * 32 + lane;
  } else if constexpr (G == 2) {
    const int g = lane >> 1;
    L.role = lane & 1;
    L.base = g * 2;
    L.gmask = 0x3u << L.base;
    traj = warp * 16 + g;
  } else if constexpr (G == 6) {
    if (lane >= 30) return false;
    const int g = lane / 6;
    L.role = lane % 6;
    L.base = g * 6;
    L.gmask = 0x3Fu << L.base;
    traj = warp * 5 + g;
  } else if constexpr (G == 14) {
    if (lane >= 28) return false;
    const int g = lane / 14;
    L.role = lane % 14;
    L.base = g * 14;
    L.gmask = 0x3FFFu << L.base;
    traj = warp * 2 + g;
    gat.slot = sm_gather + ((threadIdx.x >> 5) * 2 + g) * 84;
  } else {
    if (lane >= 28) return false;
    const int g = lane / 7;
    L.role = lane % 7;
    L.base = g * 7;
    L.gmask = 0x7Fu << L.base;
    traj = warp * 4 + g;
    gat.slot = sm_gather + ((threadIdx.x >> 5) * 4 + g) * 84;
  }
  return true;
}

// Shared-memory doubles a block of up to four warps needs for the 42-vector
// norm (one 42-double slot per lane group).
template <int G>
__host__ __device__ constexpr int gather_smem_doubles() {
  return G == 7 ? 4 * 4 * 84 : (G == 14 ? 4 * 2 * 84 : 1);
}

template <int G>
__device__ __forceinline__ bool is_leader(const Layout<G>& L) {
  return (G == 1) || ((G == 2 || G == 6 || G == 14) && L.role == 0) || (G == 7 && L.role == 6);
}

// Where the event component lives in a group: its register index r on the
// owning lane (mine), and the owning lane, which broadcasts g to the group.
template <int G>
struct EvCtx {
  int r = 0;
  bool mine = false;
  int src = 0;
  unsigned gmask = 0;
  __device__ __forceinline__ EvCtx(const Layout<G>& L, int index) {
    if (index < 0) return;
    r = L.local(index);
    if constexpr (G == 1) {
      mine = true;
    } else {
      mine = (L.role == L.owner(index));
      src = L.base + L.owner(index);
      gmask = L.gmask;
    }
  }
  __device__ __forceinline__ double bcast(double v) const {
    if constexpr (G == 1)
      return v;
    else
      return __shfl_sync(gmask, v, src);
  }
};

// _dop853_refine_in_step: bisection for the crossing on the step's dense
// interpolant (rows F, step size h, g at the step start g_left); returns the
// crossing as a fraction x of the step.
template <int G>
__device__ __forceinline__ double refine_in_step(const EvCtx<G>& ev, const double (&y)[Layout<G>::NC],
                                                 const double (&F)[7][Layout<G>::NC], double h, double g_left,
                                                 const DopParams& p) {
  constexpr int NC = Layout<G>::NC;
  double fe[7];
#pragma unroll
  for (int i = 0; i < 7; ++i) fe[i] = pick<NC>(F[i], ev.r);
  const double ye = pick<NC>(y, ev.r);
  double a = 0.0, b = 1.0;
  double x_hit = -1.0;
  for (int it = 0; it < 128; ++it) {
    const double mid = 0.5 * (a + b);
    const double g_mid = ev.bcast(ev.mine ? (DopLane<G>::eval_row(ye, fe, mid) - p.ev_offset) : 0.0);
    if (fabs(g_mid) <= p.gtol) {
      x_hit = mid;
      break;
    }
    if (crossed_direction(g_left, g_mid, p.ev_dir)) {
      b = mid;
    } else {
      a = mid;
      g_left = g_mid;
    }
    if ((b - a) * fabs(h) <= p.xtol) break;
  }
  if (x_hit < 0.0) x_hit = b;
  return x_hit;
}

// A crossing step saved for deferred refinement, structure of arrays with
// stride rec_ld: y (D), y_new (D), k[0..12] (13 D), h, t, g_left.
template <int G>
__device__ __forceinline__ int leader_lane(const Layout<G>& L) {
  if constexpr (G == 1)
    return threadIdx.x & 31;
  else if constexpr (G == 7)
    return L.base + 6;
  else
    return L.base;
}

template <int G>
__device__ __forceinline__ void save_step(const Layout<G>& L, const DopParams& p, int traj, int hit, bool leader,
                                          const double (&y)[Layout<G>::NC], const double (&yh)[Layout<G>::NC],
                                          const double (&k)[13][Layout<G>::NC], double h, double t, double g_left) {
  constexpr int D = Layout<G>::D;
  constexpr int NC = Layout<G>::NC;
  int slot = 0;
  if (leader) slot = atomicAdd(p.refine_count, 1);
  if constexpr (G > 1) slot = __shfl_sync(L.gmask, slot, leader_lane<G>(L));
  double* r = p.rec + slot;
  const long long ld = p.rec_ld;
#pragma unroll
  for (int d = 0; d < NC; ++d) {
    const int c = L.comp(d);
    r[c * ld] = y[d];
    r[(D + c) * ld] = yh[d];
#pragma unroll
    for (int j = 0; j < 13; ++j) r[(2 * D + j * D + c) * ld] = k[j][d];
  }
  if (leader) {
    r[(15 * D) * ld] = h;
    r[(15 * D + 1) * ld] = t;
    r[(15 * D + 2) * ld] = g_left;
    p.refine_list[slot] = traj;
    p.refine_hit[slot] = hit;
  }
}

// Refinement of the saved crossings, all lanes in lock step: the same dense
// cache, bisection and interpolation as the inline path.
template <int G>
__global__ void __launch_bounds__(128) refine_kernel(DopParams p) {
  constexpr int D = Layout<G>::D;
  constexpr int NC = Layout<G>::NC;
  Layout<G> L;
  Gather<G> gat;
  int slot;
  __shared__ double sm_gather[gather_smem_doubles<G>()];
  if (!setup_layout<G>(L, gat, sm_gather, slot)) return;
  const bool leader = is_leader<G>(L);
  const EvCtx<G> ev(L, p.ev_index);
  const int n = *p.refine_count;
  for (; slot < n; slot += p.stride) {
    const int traj = p.refine_list[slot];
    const int hit = p.refine_hit[slot];
    const double* r = p.rec + slot;
    const long long ld = p.rec_ld;
    double y[NC], yh[NC], k[13][NC];
#pragma unroll
    for (int d = 0; d < NC; ++d) {
      const int c = L.comp(d);
      y[d] = r[c * ld];
      yh[d] = r[(D + c) * ld];
#pragma unroll
      for (int j = 0; j < 13; ++j) k[j][d] = r[(2 * D + j * D + c) * ld];
    }
    const double h = r[(15 * D) * ld];
    const double t = r[(15 * D + 1) * ld];
    const double g_left = r[(15 * D + 2) * ld];
    double F[7][NC];
    DopLane<G>::dense_cache(L, y, yh, h, p.mu, p.dir, k, F);
    const double x_hit = refine_in_step<G>(ev, y, F, h, g_left, p);
    if (leader) p.hit_t[(long long)hit * p.ld + traj] = t + x_hit * h;
    double* o = p.hit_y + (long long)hit * D * p.ld;
#pragma unroll
    for (int d = 0; d < NC; ++d) o[(long long)L.comp(d) * p.ld + traj] = DopLane<G>::eval1(y[d], F, d, x_hit);
  }
}

// DENSE = false compiles the dense-output path out (launches without
// samples): fewer live registers in the step loop.
template <int G, bool DENSE = true>
__global__ void __launch_bounds__(128) dop853_kernel(DopParams p) {
  constexpr int D = Layout<G>::D;
  constexpr int NC = Layout<G>::NC;
  Layout<G> L;
  Gather<G> gat;
  int traj;
  __shared__ double sm_gather[gather_smem_doubles<G>()];  // 4 warps x 4 groups
  __shared__ double sm_coef[dop_spread_coef<G>() ? dop_nnz() : 1];
  if constexpr (dop_spread_coef<G>()) {
    dop_coef_table_init(sm_coef);
    __syncthreads();
  }
  if (!setup_layout<G>(L, gat, sm_gather, traj)) return;
  const bool leader = is_leader<G>(L);
  const bool has_event = p.ev_index >= 0 && p.max_hits > 0;
  const EvCtx<G> ev(L, has_event ? p.ev_index : -1);
  auto cf = dop_coef<G>(L, sm_coef);

  const int slot0 = traj;
  int slot = traj;
  while (true) {
    // attempted-step budget of this slot in a segmented launch: a lane (group)
    // holds slots slot0, slot0 + stride, ...; one with fewer slots than the
    // busiest lane (M of them) gives its last slot the difference, so every
    // lane spends the M * seg_steps steps its warp runs anyway (a warp's FP64
    // instructions cost the same whatever lanes are active) and the
    // trajectories advance further; pausing and resuming keep every bit.
    int seg_budget = p.seg_steps;
    if (p.seg) {
      const int n_in = *p.n_in;
      if (slot >= n_in) break;
      traj = p.active_in[slot];
      if (slot + p.stride >= n_in) {
        const int busiest = (n_in + p.stride - 1) / p.stride;
        seg_budget = p.seg_steps * (busiest - (slot - slot0) / p.stride);
      }
    } else if (traj >= p.N) {
      break;
    }
    const double t0 = p.t0_arr ? p.t0_arr[traj] : p.t0;
    const double tmax = p.tmax_arr ? p.tmax_arr[traj] : p.tmax;
    const bool resume = p.seg && p.status[traj] == HG_RUNNING;
    double y[NC];
    if (resume) {
#pragma unroll
      for (int r = 0; r < NC; ++r) y[r] = p.y_end[(long long)L.comp(r) * p.ld + traj];
    } else {
#pragma unroll
      for (int r = 0; r < NC; ++r) y[r] = p.y0[(long long)L.comp(r) * p.ld + traj];
    }
    double k[13][NC];
    // on resume this is bitwise k[12] of the last accepted step
    L.rhs(y, p.mu, p.dir, k[0]);
    double g_prev = 0.0;
    if (has_event) g_prev = ev.bcast(ev.mine ? (pick<NC>(y, ev.r) - p.ev_offset) : 0.0);
    double h, t, err_prev, prev_pow;
    int acc, rej, hits, q_next;
    const bool dense = DENSE && p.m >= 2;
    if (resume) {
      h = p.ws_h[traj];
      t = p.t_end[traj];
      err_prev = p.ws_err_prev[traj];
      prev_pow = p.ws_prev_pow[traj];
      acc = p.n_accept[traj];
      rej = p.n_reject[traj];
      hits = (has_event && p.n_hits) ? p.n_hits[traj] : 0;
      q_next = dense ? p.ws_q[traj] : 0;
    } else {
      double a[NC], b[NC];
#pragma unroll
      for (int d = 0; d < NC; ++d) {
        const double scale0 = p.atol + p.rtol * fabs(y[d]);
        a[d] = y[d] / scale0;
        b[d] = k[0][d] / scale0;
      }
      const double sn = sqrt((double)D);
      double na, nb;
      gat.dot2(L, a, b, na, nb);
      const double d0 = sqrt(na) / sn;
      const double d1 = sqrt(nb) / sn;
      h = select_initial_step(d0, d1, p.min_step, p.max_step);
      t = t0;
      err_prev = -1.0;
      prev_pow = 0.0;
      acc = rej = hits = 0;
      q_next = (dense && p.dense_last) ? p.m - 1 : 0;
    }
    int status = HG_OK;
    // dense sampling on linspace(t0, tmax, m)
    double step_ls = 0.0;
    if (dense) step_ls = (tmax - t0) / (double)(p.m - 1);
    auto sample_t = [&](int q) -> double { return q == p.m - 1 ? tmax : (double)q * step_ls + t0; };
    int seg_count = 0;
    bool paused = false;

    // integrators/rk.py loop test (t - t_end) * direction < 0 with direction
    // +1; the product by 1 is exact, so it is left out
    while (hg_lt0(t - tmax)) {
      if (p.seg && seg_count >= seg_budget) {
        paused = true;
        break;
      }
      ++seg_count;
      if ((long long)(acc + rej) >= p.max_steps) {
        status = HG_MAX_STEPS;
        break;
      }
      h = clamp_step(h, p.max_step, p.min_step);
      h = adjust_step_to_endpoint(t, h, tmax);
      double yh[NC], e5[NC], e3[NC];
      cf.set_step(h);
      DopLane<G>::step(L, y, cf, h, p.mu, p.dir, k, yh, e5, e3);
      double err_norm;
      {
        double s5[NC], s3[NC];
#pragma unroll
        for (int d = 0; d < NC; ++d) {
          const double scale = p.atol + p.rtol * np_maximum_abs(y[d], yh[d]);
          const double is = hg_rcp_rn(scale);
          s5[d] = hg_div_rn(e5[d], scale, is);
          s3[d] = hg_div_rn(e3[d], scale, is);
        }
        double n5, n3;
        gat.dot2(L, s5, s3, n5, n3);
        if (hg_both0(n5, n3))
          err_norm = 0.0;
        else
          err_norm = (fabs(h) * n5) / sqrt((n5 + 0.01 * n3) * (double)D);
      }
      const bool accepted = hg_le_pos(err_norm, HG_BITS_1);  // err_norm <= 1
      bool fin = true;
      if (accepted) {
        ++acc;
        const double t_new = t + h;
        bool stop = false;
        // dense samples inside (t, t_new] (reference: searchsorted on nodes)
        if (dense) {
          const bool last = !(t_new - tmax < 0.0);
          if (q_next < p.m && (last || sample_t(q_next) < t_new)) {
            const double hseg = t_new - t;
            double F[7][NC];
            DopLane<G>::dense_cache(L, y, yh, hseg, p.mu, p.dir, k, F);
            while (q_next < p.m && (last || sample_t(q_next) < t_new)) {
              const double x = (sample_t(q_next) - t) / hseg;
              double* o = p.y_out + (long long)(p.dense_last ? 0 : q_next) * D * p.ld;
#pragma unroll
              for (int d = 0; d < NC; ++d)
                o[(long long)L.comp(d) * p.ld + traj] = DopLane<G>::eval1(y[d], F, d, x);
              ++q_next;
            }
          }
        }
        if (has_event) {
          const double g_new = ev.bcast(ev.mine ? (pick<NC>(yh, ev.r) - p.ev_offset) : 0.0);
          if (event_crossed(g_prev, g_new, p.ev_dir)) {
            if (p.rec) {
              // keep the step for refine_kernel
              save_step<G>(L, p, traj, hits, leader, y, yh, k, h, t, g_prev);
            } else {
              // _dop853_refine_in_step with the step size h
              double F[7][NC];
              DopLane<G>::dense_cache(L, y, yh, h, p.mu, p.dir, k, F);
              const double x_hit = refine_in_step<G>(ev, y, F, h, g_prev, p);
              p.hit_t[(long long)hits * p.ld + traj] = t + x_hit * h;
              double* o = p.hit_y + (long long)hits * D * p.ld;
#pragma unroll
              for (int d = 0; d < NC; ++d)
                o[(long long)L.comp(d) * p.ld + traj] = DopLane<G>::eval1(y[d], F, d, x_hit);
            }
            ++hits;
            if (hits >= p.max_hits) stop = true;
          }
          g_prev = g_new;
        }
        t = t_new;
#pragma unroll
        for (int d = 0; d < NC; ++d) {
          y[d] = yh[d];
          k[0][d] = k[12][d];
          fin = fin && finite_bits(yh[d]);
        }
        if (stop) break;
      } else {
        ++rej;
      }
      h = h * pi_factor(L, accepted, err_norm, err_prev, prev_pow);
      if (accepted) {
        err_prev = err_norm;
        if constexpr (G > 1) fin = __all_sync(L.gmask, fin);
        if (!fin) {
          status = HG_NONFINITE;
          break;
        }
      } else {
        h = clamp_step(h, p.max_step, p.min_step);
      }
    }
    // outputs
    if (p.y_end) {
#pragma unroll
      for (int d = 0; d < NC; ++d) p.y_end[(long long)L.comp(d) * p.ld + traj] = y[d];
    }
    if (paused) {
      if (leader) {
        p.t_end[traj] = t;
        p.ws_h[traj] = h;
        p.ws_err_prev[traj] = err_prev;
        p.ws_prev_pow[traj] = prev_pow;
        if (dense) p.ws_q[traj] = q_next;
        if (p.n_hits) p.n_hits[traj] = hits;
        p.n_accept[traj] = acc;
        p.n_reject[traj] = rej;
        p.status[traj] = HG_RUNNING;
        p.active_out[atomicAdd(p.n_out, 1)] = traj;
      }
      slot += p.stride;
      continue;
    }
    if (dense) {
      // the reference's dense output falls back to the single stored node
      // when no step was taken
      while (q_next < p.m) {
        double* o = p.y_out + (long long)(p.dense_last ? 0 : q_next) * D * p.ld;
#pragma unroll
        for (int d = 0; d < NC; ++d) o[(long long)L.comp(d) * p.ld + traj] = y[d];
        ++q_next;
      }
    }
    if (leader) {
      if (p.t_end) p.t_end[traj] = t;
      if (p.n_hits) p.n_hits[traj] = hits;
      if (p.n_accept) p.n_accept[traj] = acc;
      if (p.n_reject) p.n_reject[traj] = rej;
      if (p.status) p.status[traj] = status;
    }
    // next trajectory
    if (p.seg) {
      slot += p.stride;
      continue;
    }
    if (p.next_traj == nullptr) break;
    int nt = 0;
    if constexpr (G == 1) {
      nt = atomicAdd(p.next_traj, 1) + p.stride;
    } else {
      if (L.role == 0) nt = atomicAdd(p.next_traj, 1) + p.stride;
      nt = __shfl_sync(L.gmask, nt, L.base);
    }
    traj = nt;
  }
}

}  // namespace hg
