/*
 * CPU oracle: operation-for-operation restatement of the reference's
 * CR3BP propagation kernels.  Test infrastructure only (see hgo.h).
 * Build with -O2 -ffp-contract=off so that no multiply-add is fused
 * behind our back; the fused operations below are explicit fma() calls
 * that mirror numpy's float64 dot.
 */
#include "hgo.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "hgo_tableaux.h"

#if defined(__aarch64__)
typedef long double hgo_quad; /* IEEE binary128 on aarch64 Linux */
#define HGO_QPOW powl
#else
#include <quadmath.h>
typedef __float128 hgo_quad;
#define HGO_QPOW powq
#endif

#define MAXD 42

static int g_mode = HGO_MODE_PYTHON;

void hgo_set_mode(int mode) { g_mode = mode; }
int hgo_get_mode(void) { return g_mode; }

double hgo_fpow(double x, double y) {
  if (g_mode == HGO_MODE_DEVICE) {
    if (!(x > 0.0) || !isfinite(x) || !isfinite(y)) return pow(x, y);
    return (double)HGO_QPOW((hgo_quad)x, (hgo_quad)y);
  }
  return pow(x, y);
}

double hgo_ipow2(double x) {
  if (g_mode == HGO_MODE_PYTHON) return pow(x, 2.0);
  return x * x;
}

double hgo_ipow3(double x) {
  if (g_mode == HGO_MODE_PYTHON) return pow(x, 3.0);
  return x * (x * x);
}

/* ---------------------------------------------------------------------------
 * Vector fields
 * ------------------------------------------------------------------------- */

/* dynamics/rtbp.py:30-74 (_crtbp_accel) */
void hgo_rhs6(const double* s, double mu, double* d) {
  const double x = s[0], y = s[1], z = s[2], vx = s[3], vy = s[4], vz = s[5];
  const double r1 = sqrt((hgo_ipow2(x + mu) + hgo_ipow2(y)) + hgo_ipow2(z));
  const double r2 = sqrt((hgo_ipow2(x - (1 - mu)) + hgo_ipow2(y)) + hgo_ipow2(z));
  const double r1c = hgo_ipow3(r1);
  const double r2c = hgo_ipow3(r2);
  const double ax = ((2 * vy + x) - ((1 - mu) * (x + mu)) / r1c) - (mu * ((x - 1) + mu)) / r2c;
  const double ay = ((-2 * vx + y) - ((1 - mu) * y) / r1c) - (mu * y) / r2c;
  const double az = ((-(1 - mu)) * z) / r1c - (mu * z) / r2c;
  d[0] = vx;
  d[1] = vy;
  d[2] = vz;
  d[3] = ax;
  d[4] = ay;
  d[5] = az;
}

/* dynamics/rtbp.py:76-165 (_jacobian_crtbp) and :167-255 (_var_equations).
 * Phi = y[0:36] row-major, state = y[36:42]. */
void hgo_rhs42(const double* Y, double mu, double* D) {
  const double* P = Y;
  const double x = Y[36], y = Y[37], z = Y[38], vx = Y[39], vy = Y[40], vz = Y[41];

  /* _jacobian_crtbp */
  const double mu2 = 1.0 - mu;
  double r2 = (hgo_ipow2(x + mu) + hgo_ipow2(y)) + hgo_ipow2(z);
  double R2 = (hgo_ipow2(x - mu2) + hgo_ipow2(y)) + hgo_ipow2(z);
  double r3 = hgo_fpow(r2, 1.5);
  double r5 = hgo_fpow(r2, 2.5);
  double R3 = hgo_fpow(R2, 1.5);
  double R5 = hgo_fpow(R2, 2.5);
  const double c3 = mu2 / r3 + mu / R3;
  const double omgxx = ((1.0 + ((mu2 / r5) * 3.0) * hgo_ipow2(x + mu)) +
                        ((mu / R5) * 3.0) * hgo_ipow2(x - mu2)) - c3;
  const double omgyy = ((1.0 + ((mu2 / r5) * 3.0) * hgo_ipow2(y)) +
                        ((mu / R5) * 3.0) * hgo_ipow2(y)) - c3;
  const double omgzz = ((0.0 + ((mu2 / r5) * 3.0) * hgo_ipow2(z)) +
                        ((mu / R5) * 3.0) * hgo_ipow2(z)) - c3;
  const double sxy = (mu2 * (x + mu)) / r5 + (mu * (x - mu2)) / R5;
  const double omgxy = (3.0 * y) * sxy;
  const double omgxz = (3.0 * z) * sxy;
  const double omgyz = ((3.0 * y) * z) * (mu2 / r5 + mu / R5);

  double F[6][6];
  memset(F, 0, sizeof(F));
  F[0][3] = 1.0;
  F[1][4] = 1.0;
  F[2][5] = 1.0;
  F[3][0] = omgxx; F[3][1] = omgxy; F[3][2] = omgxz;
  F[4][0] = omgxy; F[4][1] = omgyy; F[4][2] = omgyz;
  F[5][0] = omgxz; F[5][1] = omgyz; F[5][2] = omgzz;
  F[3][4] = 2.0;
  F[4][3] = -2.0;

  for (int i = 0; i < 6; ++i) {
    for (int j = 0; j < 6; ++j) {
      double acc = 0.0;
      for (int k = 0; k < 6; ++k) acc += F[i][k] * P[6 * k + j];
      D[6 * i + j] = acc;
    }
  }

  /* state part of _var_equations (recomputes r2, R2, r3, R3) */
  r2 = (hgo_ipow2(x + mu) + hgo_ipow2(y)) + hgo_ipow2(z);
  R2 = (hgo_ipow2(x - mu2) + hgo_ipow2(y)) + hgo_ipow2(z);
  r3 = hgo_fpow(r2, 1.5);
  R3 = hgo_fpow(R2, 1.5);
  const double ax = ((x - mu2 * ((x + mu) / r3)) - mu * ((x - mu2) / R3)) + 2.0 * vy;
  const double ay = ((y - mu2 * (y / r3)) - mu * (y / R3)) - 2.0 * vx;
  const double az = (-mu2) * (z / r3) - mu * (z / R3);
  D[36] = vx;
  D[37] = vy;
  D[38] = vz;
  D[39] = ax;
  D[40] = ay;
  D[41] = az;
}

typedef struct {
  int dim;
  double mu;
  int fwd;
  int flo, fhi;
} hgo_sys;

/* dynamics/base.py:272-310: negate the flipped components for fwd = -1 */
static void sys_rhs(const hgo_sys* S, const double* y, double* dy) {
  if (S->dim == 6)
    hgo_rhs6(y, S->mu, dy);
  else
    hgo_rhs42(y, S->mu, dy);
  if (S->fwd == -1) {
    for (int i = S->flo; i < S->fhi; ++i) dy[i] = -dy[i];
  }
}

/* ---------------------------------------------------------------------------
 * numpy float64 dot / norm order (see header)
 * ------------------------------------------------------------------------- */
static double np_dot_self(const double* v, int n) {
  int i = 0;
  double dot = 0.0;
  if (n >= 32) {
    /* only n == 42 is used: one 32-element block */
    double p[32];
    for (int q = 0; q < 32; ++q) p[q] = v[q] * v[q];
    double a[4][4];
    for (int k = 0; k < 4; ++k)
      for (int m = 0; m < 4; ++m) a[k][m] = p[8 * k + m] + p[8 * k + 4 + m];
    double s[4];
    for (int m = 0; m < 4; ++m) s[m] = ((a[0][m] + a[1][m]) + a[2][m]) + a[3][m];
    dot = (s[0] + s[2]) + (s[1] + s[3]);
    i = 32;
  }
  for (; i < n; ++i) dot = fma(v[i], v[i], dot);
  return dot;
}

/* ---------------------------------------------------------------------------
 * Step-size helpers, integrators/utils.py:126-296
 * ------------------------------------------------------------------------- */
static double select_initial_step(double d0, double d1, double min_step, double max_step) {
  double h;
  if (d0 < 1.0e-5 || d1 < 1.0e-5)
    h = 1.0e-6;
  else
    h = (0.01 * d0) / d1;
  if (h > max_step) h = max_step;
  if (h < min_step) h = min_step;
  return h;
}

static double clamp_step(double h, double max_step, double min_step) {
  if (h > max_step) h = max_step;
  if (h < min_step) h = min_step;
  return h;
}

static double adjust_step_to_endpoint(double t, double h, double t_end) {
  if (t + h > t_end) return fabs(t_end - t);
  return h;
}

static double pi_accept_factor(double err_norm, double err_prev, double order) {
  const double beta = 1.0 / (order + 1.0);
  const double alpha = 0.4 * beta;
  double factor;
  if (err_prev < 0.0) {
    if (err_norm == 0.0)
      factor = 10.0;
    else
      factor = 0.9 * hgo_fpow(err_norm, -beta);
  } else {
    if (err_norm == 0.0)
      factor = 10.0;
    else
      factor = (0.9 * hgo_fpow(err_norm, -beta)) * hgo_fpow(err_prev, alpha);
  }
  if (!(factor == factor)) factor = 10.0;
  if (factor < 0.2) factor = 0.2;
  if (factor > 10.0) factor = 10.0;
  return factor;
}

static double pi_reject_factor(double err_norm, double order) {
  const double err_exp = 1.0 / order;
  double factor;
  if (err_norm <= 0.0)
    factor = 0.2;
  else
    factor = 0.9 * hgo_fpow(err_norm, -err_exp);
  if (!(factor == factor)) factor = 0.2;
  if (factor < 0.2) factor = 0.2;
  if (factor > 10.0) factor = 10.0;
  return factor;
}

/* integrators/utils.py:13-39 */
static int event_crossed(double g_prev, double g_new, int direction) {
  if (direction == 0)
    return (g_prev < 0.0 && g_new > 0.0) || (g_prev > 0.0 && g_new < 0.0) || (g_new == 0.0);
  else if (direction > 0)
    return (g_prev < 0.0 && g_new > 0.0) || (g_new == 0.0);
  else
    return (g_prev > 0.0 && g_new < 0.0) || (g_new == 0.0);
}

/* integrators/utils.py:42-68 */
static int crossed_direction(double g_left, double g_mid, int direction) {
  if (direction == 0)
    return (g_left < 0.0 && g_mid > 0.0) || (g_left > 0.0 && g_mid < 0.0);
  else if (direction > 0)
    return (g_left < 0.0 && g_mid > 0.0);
  else
    return (g_left > 0.0 && g_mid < 0.0);
}

static double np_maximum(double a, double b) {
  if (isnan(a) || isnan(b)) return NAN;
  return a >= b ? a : b;
}

/* ---------------------------------------------------------------------------
 * Fixed-step RK, integrators/rk.py:154-215 and :531-588
 * ------------------------------------------------------------------------- */
typedef struct {
  int s;
  const double* A; /* s x s row-major */
  const double* B;
} hgo_tab;

static int get_fixed_tab(int order, hgo_tab* T) {
  switch (order) {
    case 4: T->s = 4; T->A = &HGO_RK4_A[0][0]; T->B = HGO_RK4_B; return 1;
    case 6: T->s = 7; T->A = &HGO_RK6_A[0][0]; T->B = HGO_RK6_B; return 1;
    case 8: T->s = 13; T->A = &HGO_RK8_A[0][0]; T->B = HGO_RK8_B; return 1;
    default: return 0;
  }
}

static void rk_step(const hgo_sys* S, const hgo_tab* T, const double* y, double h,
                    double k[][MAXD], double* y_high) {
  const int n = S->dim;
  double ys[MAXD];
  sys_rhs(S, y, k[0]);
  for (int i = 1; i < T->s; ++i) {
    memcpy(ys, y, sizeof(double) * n);
    for (int j = 0; j < i; ++j) {
      const double a = T->A[i * T->s + j];
      if (a != 0.0) {
        const double c = h * a;
        for (int d = 0; d < n; ++d) ys[d] = ys[d] + c * k[j][d];
      }
    }
    sys_rhs(S, ys, k[i]);
  }
  memcpy(y_high, y, sizeof(double) * n);
  for (int j = 0; j < T->s; ++j) {
    const double b = T->B[j];
    if (b != 0.0) {
      const double c = h * b;
      for (int d = 0; d < n; ++d) y_high[d] = y_high[d] + c * k[j][d];
    }
  }
}

static int all_finite(const double* v, int n) {
  for (int i = 0; i < n; ++i)
    if (!isfinite(v[i])) return 0;
  return 1;
}

int hgo_fixed_rk(int order, int dim, double mu, int fwd, int flip_lo, int flip_hi,
                 const double* y0, const double* t_vals, int n, double* states) {
  hgo_tab T;
  if (!get_fixed_tab(order, &T) || (dim != 6 && dim != 42) || n < 1) return HGO_BAD_ARGS;
  hgo_sys S = {dim, mu, fwd, flip_lo, flip_hi};
  double k[13][MAXD];
  memcpy(states, y0, sizeof(double) * dim);
  int status = HGO_OK;
  for (int idx = 0; idx < n - 1; ++idx) {
    const double h = t_vals[idx + 1] - t_vals[idx];
    rk_step(&S, &T, states + (size_t)idx * dim, h, k, states + (size_t)(idx + 1) * dim);
    if (status == HGO_OK && !all_finite(states + (size_t)(idx + 1) * dim, dim)) status = HGO_NONFINITE;
  }
  return status;
}

/* ---------------------------------------------------------------------------
 * DOP853, integrators/rk.py:1636-1708 (step), :1790-2003 (dense output)
 * ------------------------------------------------------------------------- */
#define NS HGO_DOP_N_STAGES     /* 12 */
#define NSE HGO_DOP_N_STAGES_EXT /* 16 */
#define IP HGO_DOP_INTERP_POWER  /* 7 */

/* One DOP853 step.  k has 13 rows (k[12] = f(t+h, y_high)). */
static void dop853_step(const hgo_sys* S, const double* y, double h, double k[][MAXD],
                        double* y_high, double* err5, double* err3) {
  const int n = S->dim;
  double ys[MAXD];
  sys_rhs(S, y, k[0]);
  for (int i = 1; i < NS; ++i) {
    memcpy(ys, y, sizeof(double) * n);
    for (int j = 0; j < i; ++j) {
      const double a = HGO_DOP_A[i][j];
      if (a != 0.0) {
        const double c = h * a;
        for (int d = 0; d < n; ++d) ys[d] = ys[d] + c * k[j][d];
      }
    }
    sys_rhs(S, ys, k[i]);
  }
  memcpy(y_high, y, sizeof(double) * n);
  for (int j = 0; j < NS; ++j) {
    const double b = HGO_DOP_B[j];
    if (b != 0.0) {
      const double c = h * b;
      for (int d = 0; d < n; ++d) y_high[d] = y_high[d] + c * k[j][d];
    }
  }
  sys_rhs(S, y_high, k[NS]);
  for (int d = 0; d < n; ++d) {
    err5[d] = 0.0;
    err3[d] = 0.0;
  }
  for (int j = 0; j < NS + 1; ++j) {
    const double c5 = HGO_DOP_E5[j];
    const double c3 = HGO_DOP_E3[j];
    if (c5 != 0.0)
      for (int d = 0; d < n; ++d) err5[d] = err5[d] + c5 * k[j][d];
    if (c3 != 0.0)
      for (int d = 0; d < n; ++d) err3[d] = err3[d] + c3 * k[j][d];
  }
  for (int d = 0; d < n; ++d) {
    err5[d] = err5[d] * h;
    err3[d] = err3[d] * h;
  }
}

/* the combined error norm of rk.py:2457-2467 */
static double dop853_err_norm(int n, const double* y, const double* y_high, const double* err5,
                              const double* err3, double h, double rtol, double atol) {
  double e5[MAXD], e3[MAXD];
  for (int d = 0; d < n; ++d) {
    const double scale = atol + rtol * np_maximum(fabs(y[d]), fabs(y_high[d]));
    e5[d] = err5[d] / scale;
    e3[d] = err3[d] / scale;
  }
  const double n5 = np_dot_self(e5, n);
  const double n3 = np_dot_self(e3, n);
  if (n5 == 0.0 && n3 == 0.0) return 0.0;
  const double denom = n5 + 0.01 * n3;
  return (fabs(h) * n5) / sqrt(denom * (double)n);
}

/* initial-step heuristic, rk.py:2396-2401 / :2750-2756 */
static double dop853_initial_step(int n, const double* y, const double* f0, double rtol, double atol,
                                  double min_step, double max_step) {
  double a[MAXD], b[MAXD];
  for (int d = 0; d < n; ++d) {
    const double scale0 = atol + rtol * fabs(y[d]);
    a[d] = y[d] / scale0;
    b[d] = f0[d] / scale0;
  }
  const double sn = sqrt((double)n);
  const double d0 = sqrt(np_dot_self(a, n)) / sn;
  const double d1 = sqrt(np_dot_self(b, n)) / sn;
  return select_initial_step(d0, d1, min_step, max_step);
}

/* _dop853_build_dense_cache, rk.py:1790-1875.  K: the step's 13 stages. */
static void dop853_dense_cache(const hgo_sys* S, const double* y_old, const double* f_old,
                               const double* y_new, const double* f_new, double hseg,
                               double K[][MAXD], double F[][MAXD]) {
  const int n = S->dim;
  double Kext[NSE][MAXD];
  for (int r = 0; r < NS + 1; ++r) memcpy(Kext[r], K[r], sizeof(double) * n);
  double ys[MAXD];
  for (int srow = NS + 1; srow < NSE; ++srow) {
    for (int d = 0; d < n; ++d) {
      double acc = 0.0;
      for (int r = 0; r < srow; ++r) {
        const double a = HGO_DOP_A[srow][r];
        if (a != 0.0) acc = acc + a * Kext[r][d];
      }
      ys[d] = y_old[d] + hseg * acc;
    }
    sys_rhs(S, ys, Kext[srow]);
  }
  for (int d = 0; d < n; ++d) {
    const double dy = y_new[d] - y_old[d];
    F[0][d] = dy;
    F[1][d] = hseg * f_old[d] - dy;
    F[2][d] = 2.0 * dy - hseg * (f_new[d] + f_old[d]);
  }
  for (int irem = 0; irem < IP - 3; ++irem) {
    for (int d = 0; d < n; ++d) {
      double acc = 0.0;
      for (int r = 0; r < NSE; ++r) {
        const double c = HGO_DOP_D[irem][r];
        if (c != 0.0) acc = acc + c * Kext[r][d];
      }
      F[3 + irem][d] = hseg * acc;
    }
  }
}

/* _dop853_eval_dense, rk.py:1961-2003, for one component */
static double dop853_eval1(double y_old, double F[][MAXD], int d, double x) {
  double v = 0.0;
  for (int i = IP - 1; i >= 0; --i) {
    v = v + F[i][d];
    if ((IP - 1 - i) % 2 == 0)
      v = v * x;
    else
      v = v * (1.0 - x);
  }
  return v + y_old;
}

static void dop853_eval(int n, const double* y_old, double F[][MAXD], double x, double* out) {
  for (int d = 0; d < n; ++d) out[d] = dop853_eval1(y_old[d], F, d, x);
}

/* _dop853_refine_in_step, rk.py:2005-2102, plane event g = y[idx] - off */
static void dop853_refine(const hgo_sys* S, int ev_idx, double ev_off, double t0, const double* y0,
                          const double* f0, const double* y1, const double* f1, double h,
                          double K[][MAXD], int direction, double xtol, double gtol,
                          double* t_hit, double* y_hit) {
  double F[IP][MAXD];
  dop853_dense_cache(S, y0, f0, y1, f1, h, K, F);
  double a = 0.0, b = 1.0;
  double g_left = y0[ev_idx] - ev_off;
  for (int it = 0; it < 128; ++it) {
    const double mid = 0.5 * (a + b);
    const double g_mid = dop853_eval1(y0[ev_idx], F, ev_idx, mid) - ev_off;
    if (fabs(g_mid) <= gtol) {
      *t_hit = t0 + mid * h;
      dop853_eval(S->dim, y0, F, mid, y_hit);
      return;
    }
    if (crossed_direction(g_left, g_mid, direction)) {
      b = mid;
    } else {
      a = mid;
      g_left = g_mid;
    }
    if ((b - a) * fabs(h) <= xtol) break;
  }
  *t_hit = t0 + b * h;
  dop853_eval(S->dim, y0, F, b, y_hit);
}

int hgo_dop853_event(int dim, double mu, int fwd, int flip_lo, int flip_hi, const double* y0,
                     double t0, double tmax, double rtol, double atol, double max_step,
                     double min_step, long max_steps, int ev_index, double ev_offset, int ev_dir,
                     int max_hits, double xtol, double gtol, double* hit_t, double* hit_y,
                     int* n_hits, double* t_end, double* y_end, long* n_accept, long* n_reject) {
  if ((dim != 6 && dim != 42) || ev_index < 0 || ev_index >= dim || max_hits < 0) return HGO_BAD_ARGS;
  hgo_sys S = {dim, mu, fwd, flip_lo, flip_hi};
  double y[MAXD], f_curr[MAXD], y_high[MAXD], err5[MAXD], err3[MAXD];
  double K[NS + 1][MAXD];
  double t = t0;
  memcpy(y, y0, sizeof(double) * dim);
  sys_rhs(&S, y, f_curr);
  double g_prev = y[ev_index] - ev_offset;
  double h = dop853_initial_step(dim, y, f_curr, rtol, atol, min_step, max_step);
  double err_prev = -1.0;
  long acc = 0, rej = 0;
  int hits = 0;
  int status = HGO_OK;
  while ((t - tmax) * 1.0 < 0.0) {
    if (acc + rej >= max_steps) {
      status = HGO_MAX_STEPS;
      break;
    }
    h = clamp_step(h, max_step, min_step);
    h = adjust_step_to_endpoint(t, h, tmax);
    dop853_step(&S, y, h, K, y_high, err5, err3);
    const double err_norm = dop853_err_norm(dim, y, y_high, err5, err3, h, rtol, atol);
    if (err_norm <= 1.0) {
      ++acc;
      const double t_new = t + h;
      const double g_new = y_high[ev_index] - ev_offset;
      if (max_hits > 0 && event_crossed(g_prev, g_new, ev_dir)) {
        dop853_refine(&S, ev_index, ev_offset, t, y, f_curr, y_high, K[NS], h, K, ev_dir, xtol,
                      gtol, &hit_t[hits], &hit_y[(size_t)hits * dim]);
        ++hits;
        if (hits >= max_hits) {
          t = t_new;
          memcpy(y, y_high, sizeof(double) * dim);
          break;
        }
      }
      t = t_new;
      memcpy(y, y_high, sizeof(double) * dim);
      memcpy(f_curr, K[NS], sizeof(double) * dim);
      g_prev = g_new;
      h = h * pi_accept_factor(err_norm, err_prev, 8.0);
      err_prev = err_norm;
      if (!all_finite(y, dim)) {
        status = HGO_NONFINITE;
        break;
      }
    } else {
      ++rej;
      h = h * pi_reject_factor(err_norm, 8.0);
      h = clamp_step(h, max_step, min_step);
    }
  }
  if (n_hits) *n_hits = hits;
  if (t_end) *t_end = t;
  if (y_end) memcpy(y_end, y, sizeof(double) * dim);
  if (n_accept) *n_accept = acc;
  if (n_reject) *n_reject = rej;
  return status;
}

int hgo_dop853_dense(int dim, double mu, int fwd, int flip_lo, int flip_hi, const double* y0,
                     const double* t_eval, int m, double rtol, double atol, double max_step,
                     double min_step, long max_steps, double* y_out, long* n_accept,
                     long* n_reject) {
  if ((dim != 6 && dim != 42) || m < 1) return HGO_BAD_ARGS;
  hgo_sys S = {dim, mu, fwd, flip_lo, flip_hi};
  double y[MAXD], f_curr[MAXD], y_high[MAXD], err5[MAXD], err3[MAXD];
  double K[NS + 1][MAXD];
  double F[IP][MAXD];
  const double tf = t_eval[m - 1];
  double t = t_eval[0];
  memcpy(y, y0, sizeof(double) * dim);
  sys_rhs(&S, y, f_curr);
  double h = dop853_initial_step(dim, y, f_curr, rtol, atol, min_step, max_step);
  double err_prev = -1.0;
  long acc = 0, rej = 0;
  int idx = 0;
  int status = HGO_OK;
  while ((t - tf) * 1.0 < 0.0) {
    if (acc + rej >= max_steps) {
      status = HGO_MAX_STEPS;
      break;
    }
    h = clamp_step(h, max_step, min_step);
    h = adjust_step_to_endpoint(t, h, tf);
    dop853_step(&S, y, h, K, y_high, err5, err3);
    const double err_norm = dop853_err_norm(dim, y, y_high, err5, err3, h, rtol, atol);
    if (err_norm <= 1.0) {
      ++acc;
      const double t_new = t + h;
      const int last = !((t_new - tf) * 1.0 < 0.0);
      int built = 0;
      const double hseg = t_new - t;
      while (idx < m && (last || t_eval[idx] < t_new)) {
        if (hseg == 0.0) {
          memcpy(y_out + (size_t)idx * dim, y, sizeof(double) * dim);
        } else {
          if (!built) {
            dop853_dense_cache(&S, y, f_curr, y_high, K[NS], hseg, K, F);
            built = 1;
          }
          const double x = (t_eval[idx] - t) / hseg;
          dop853_eval(dim, y, F, x, y_out + (size_t)idx * dim);
        }
        ++idx;
      }
      t = t_new;
      memcpy(y, y_high, sizeof(double) * dim);
      memcpy(f_curr, K[NS], sizeof(double) * dim);
      h = h * pi_accept_factor(err_norm, err_prev, 8.0);
      err_prev = err_norm;
      if (!all_finite(y, dim)) {
        status = HGO_NONFINITE;
        break;
      }
    } else {
      ++rej;
      h = h * pi_reject_factor(err_norm, 8.0);
      h = clamp_step(h, max_step, min_step);
    }
  }
  /* no step taken (zero or negative span): the reference falls back to
   * the single stored node */
  for (; idx < m; ++idx) memcpy(y_out + (size_t)idx * dim, y, sizeof(double) * dim);
  if (n_accept) *n_accept = acc;
  if (n_reject) *n_reject = rej;
  return status;
}

/* _hermite_eval_dense, integrators/rk.py:286-327 */
static double hermite_eval(double y0, double f0, double y1, double f1, double x, double h) {
  const double x2 = x * x;
  const double x3 = x2 * x;
  const double H00 = (2.0 * x3 - 3.0 * x2) + 1.0;
  const double H10 = (x3 - 2.0 * x2) + x;
  const double H01 = -2.0 * x3 + 3.0 * x2;
  const double H11 = x3 - x2;
  return ((H00 * y0 + H10 * (h * f0)) + H01 * y1) + H11 * (h * f1);
}

/* _integrate_fixed_rk_until_event (integrators/rk.py:655-718) with
 * _hermite_refine_in_step (:330-391); plane g = y[ev_index] - ev_offset.
 * Returns 1 on a crossing (t_hit, y_hit set), 0 otherwise; states (n, dim)
 * rows are written up to the step before the crossing. */
int hgo_fixed_rk_event(int order, int dim, double mu, int fwd, int flip_lo, int flip_hi, const double* y0,
                       const double* t_vals, int n, int ev_index, double ev_offset, int ev_dir, double xtol,
                       double gtol, double* states, double* t_hit, double* y_hit) {
  hgo_tab T;
  if (!get_fixed_tab(order, &T) || (dim != 6 && dim != 42) || n < 1) return -1;
  hgo_sys S = {dim, mu, fwd, flip_lo, flip_hi};
  double k[13][MAXD], f_prev[MAXD], f_new[MAXD], yn[MAXD];
  memcpy(states, y0, sizeof(double) * dim);
  sys_rhs(&S, y0, f_prev);
  double g_prev = y0[ev_index] - ev_offset;
  for (int idx = 0; idx < n - 1; ++idx) {
    const double t_n = t_vals[idx];
    const double h = t_vals[idx + 1] - t_n;
    const double* y = states + (size_t)idx * dim;
    rk_step(&S, &T, y, h, k, yn);
    sys_rhs(&S, yn, f_new);
    const double g_new = yn[ev_index] - ev_offset;
    if (event_crossed(g_prev, g_new, ev_dir)) {
      double a = 0.0, b = 1.0, g_left = g_prev, x_hit = -1.0;
      const int e = ev_index;
      for (int it = 0; it < 128; ++it) {
        const double mid = 0.5 * (a + b);
        const double g_mid = hermite_eval(y[e], f_prev[e], yn[e], f_new[e], mid, h) - ev_offset;
        if (fabs(g_mid) <= gtol) {
          x_hit = mid;
          break;
        }
        if (crossed_direction(g_left, g_mid, ev_dir)) {
          b = mid;
        } else {
          a = mid;
          g_left = g_mid;
        }
        if ((b - a) * fabs(h) <= xtol) break;
      }
      if (x_hit < 0.0) x_hit = b;
      *t_hit = t_n + x_hit * h;
      for (int d = 0; d < dim; ++d) y_hit[d] = hermite_eval(y[d], f_prev[d], yn[d], f_new[d], x_hit, h);
      return 1;
    }
    memcpy(states + (size_t)(idx + 1) * dim, yn, sizeof(double) * dim);
    memcpy(f_prev, f_new, sizeof(double) * dim);
    g_prev = g_new;
  }
  return 0;
}

/* ---------------------------------------------------------------------------
 * Threaded batches (one trajectory per task)
 * ------------------------------------------------------------------------- */
typedef struct {
  int kind;
  int next;
  pthread_mutex_t lock;
  /* shared arguments */
  int order, dim, fwd, flo, fhi, N, n, out_every, ev_index, ev_dir, max_hits;
  double mu, t0, tmax, rtol, atol, max_step, min_step, ev_offset, xtol, gtol;
  long max_steps;
  const double* y0;
  const double* t_vals;
  double* out;
  double *hit_t, *hit_y, *t_end, *y_end;
  int *n_hits, *status;
  long *n_accept, *n_reject;
  int rc;
} hgo_job;

static int job_take(hgo_job* J) {
  pthread_mutex_lock(&J->lock);
  const int i = J->next < J->N ? J->next++ : -1;
  pthread_mutex_unlock(&J->lock);
  return i;
}

static void* job_worker(void* arg) {
  hgo_job* J = (hgo_job*)arg;
  for (;;) {
    const int i = job_take(J);
    if (i < 0) break;
    const double* y0 = J->y0 + (size_t)i * J->dim;
    if (J->kind == 0) {
      double* states = (double*)malloc(sizeof(double) * (size_t)J->n * J->dim);
      const int st = hgo_fixed_rk(J->order, J->dim, J->mu, J->fwd, J->flo, J->fhi, y0, J->t_vals,
                                  J->n, states);
      const int n_out = (J->n - 1) / J->out_every + 1;
      for (int r = 0; r < n_out; ++r)
        memcpy(J->out + ((size_t)i * n_out + r) * J->dim, states + (size_t)r * J->out_every * J->dim,
               sizeof(double) * J->dim);
      free(states);
      if (st != HGO_OK) J->rc = st;
    } else {
      const int st = hgo_dop853_event(
          J->dim, J->mu, J->fwd, J->flo, J->fhi, y0, J->t0, J->tmax, J->rtol, J->atol, J->max_step,
          J->min_step, J->max_steps, J->ev_index, J->ev_offset, J->ev_dir, J->max_hits, J->xtol,
          J->gtol, J->hit_t + (size_t)i * (J->max_hits > 0 ? J->max_hits : 1),
          J->hit_y + (size_t)i * (J->max_hits > 0 ? J->max_hits : 1) * J->dim, J->n_hits + i,
          J->t_end + i, J->y_end + (size_t)i * J->dim, J->n_accept + i, J->n_reject + i);
      J->status[i] = st;
    }
  }
  return NULL;
}

static int run_job(hgo_job* J, int threads) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t tid[256];
  pthread_mutex_init(&J->lock, NULL);
  J->next = 0;
  J->rc = HGO_OK;
  for (int i = 0; i < threads; ++i) pthread_create(&tid[i], NULL, job_worker, J);
  for (int i = 0; i < threads; ++i) pthread_join(tid[i], NULL);
  pthread_mutex_destroy(&J->lock);
  return J->rc;
}

int hgo_fixed_rk_batch(int order, int dim, double mu, int fwd, int flip_lo, int flip_hi, int N,
                       const double* y0, const double* t_vals, int n, int out_every, double* out,
                       int threads) {
  if (out_every < 1 || n < 1 || N < 0) return HGO_BAD_ARGS;
  hgo_job J;
  memset(&J, 0, sizeof(J));
  J.kind = 0;
  J.order = order; J.dim = dim; J.mu = mu; J.fwd = fwd; J.flo = flip_lo; J.fhi = flip_hi;
  J.N = N; J.y0 = y0; J.t_vals = t_vals; J.n = n; J.out_every = out_every; J.out = out;
  return run_job(&J, threads);
}

int hgo_dop853_event_batch(int dim, double mu, int fwd, int flip_lo, int flip_hi, int N,
                           const double* y0, double t0, double tmax, double rtol, double atol,
                           double max_step, double min_step, long max_steps, int ev_index,
                           double ev_offset, int ev_dir, int max_hits, double xtol, double gtol,
                           double* hit_t, double* hit_y, int* n_hits, double* t_end, double* y_end,
                           long* n_accept, long* n_reject, int* status, int threads) {
  hgo_job J;
  memset(&J, 0, sizeof(J));
  J.kind = 1;
  J.dim = dim; J.mu = mu; J.fwd = fwd; J.flo = flip_lo; J.fhi = flip_hi; J.N = N; J.y0 = y0;
  J.t0 = t0; J.tmax = tmax; J.rtol = rtol; J.atol = atol; J.max_step = max_step;
  J.min_step = min_step; J.max_steps = max_steps; J.ev_index = ev_index; J.ev_offset = ev_offset;
  J.ev_dir = ev_dir; J.max_hits = max_hits; J.xtol = xtol; J.gtol = gtol; J.hit_t = hit_t;
  J.hit_y = hit_y; J.n_hits = n_hits; J.t_end = t_end; J.y_end = y_end; J.n_accept = n_accept;
  J.n_reject = n_reject; J.status = status;
  run_job(&J, threads);
  return HGO_OK;
}

/* ---------------------------------------------------------------------------
 * Section crossings on one sampled trajectory,
 * poincare/synodic/backend.py:458-659 (_detect_with_segment_refine) and
 * :382-455 (_order_and_dedup_hits), plane g = y[axis] - offset,
 * poincare/utils.py:53-147 (_hermite_scalar / _hermite_der, numba-compiled:
 * squares through hgo_ipow2 outside PYTHON mode; the state interpolation in
 * backend.py is plain Python, so its squares are libm pow except in DEVICE
 * mode).  times/states are (m,) and (m, 6) row-major.  Returns the number of
 * accepted hits (all of them); stores at most max_hits.
 * ------------------------------------------------------------------------- */
static double sq_py(double x) { return g_mode == HGO_MODE_DEVICE ? x * x : pow(x, 2.0); }

static double herm_s(double s, double y0, double y1, double dy0, double dy1, double dt) {
  const double h00 = (1.0 + 2.0 * s) * hgo_ipow2(1.0 - s);
  const double h10 = s * hgo_ipow2(1.0 - s);
  const double h01 = hgo_ipow2(s) * (3.0 - 2.0 * s);
  const double h11 = hgo_ipow2(s) * (s - 1.0);
  return ((h00 * y0 + (h10 * dy0) * dt) + h01 * y1) + (h11 * dy1) * dt;
}

static double herm_d(double s, double y0, double y1, double dy0, double dy1, double dt) {
  const double dh00 = ((6.0 * s) * (s - 1.0) + hgo_ipow2(1.0 - s) * 2.0) - (2.0 * (1.0 - s)) * (1.0 + 2.0 * s);
  const double dh10 = hgo_ipow2(1.0 - s) + s * (2.0 * (s - 1.0));
  const double dh01 = (6.0 * s) * (1.0 - s) - (2.0 * s) * (3.0 - 2.0 * s);
  const double dh11 = (2.0 * s) * (s - 1.0) + hgo_ipow2(s);
  return ((dh00 * y0 + (dh10 * dy0) * dt) + dh01 * y1) + (dh11 * dy1) * dt;
}

typedef struct {
  int have, stored, found, max_hits, pu, pv;
  double pt, pu_v, pv_v, dtt, dpt;
  double *hit_t, *hit_y;
} hgo_emit;

static int emit(hgo_emit* E, double th, const double* x) {
  if (E->max_hits > 0 && E->stored >= E->max_hits) return 1;
  const double u = x[E->pu], v = x[E->pv];
  if (E->have) {
    if (fabs(th - E->pt) <= E->dtt) return 0;
    const double du = u - E->pu_v, dv = v - E->pv_v;
    if ((du * du + dv * dv) <= (E->dpt * E->dpt)) return 0;
  }
  E->have = 1;
  E->pt = th;
  E->pu_v = u;
  E->pv_v = v;
  E->found++;
  E->hit_t[E->stored] = th;
  memcpy(E->hit_y + 6 * E->stored, x, sizeof(double) * 6);
  E->stored++;
  return E->max_hits > 0 && E->stored >= E->max_hits;
}

int hgo_section_detect(const double* times, const double* states, int m, int axis, double offset, int direction,
                       int pu, int pv, int segment_refine, int cubic, int newton_max_iter, double tol_on_surface,
                       double dedup_time_tol, double dedup_point_tol, int max_hits, double* hit_t, double* hit_y,
                       int* n_stored) {
  hgo_emit E;
  memset(&E, 0, sizeof(E));
  E.max_hits = max_hits;
  E.pu = pu;
  E.pv = pv;
  E.dtt = dedup_time_tol;
  E.dpt = dedup_point_tol;
  E.hit_t = hit_t;
  E.hit_y = hit_y;
  const int N = m, r = segment_refine;
  if (r <= 0 || N < 2) {
    *n_stored = 0;
    return 0;
  }
  const double step = 1.0 / (r + 1);
#define G(q) (states[6 * (q) + axis] - offset)
  int stop = 0;
  for (int k = 0; k < N - 1 && !stop; ++k) {
    const double t0 = times[k], t1 = times[k + 1], dt = t1 - t0;
    const double gk = G(k), gk1 = G(k + 1);
    double d0 = 0.0, d1 = 0.0;
    const int cub = cubic && dt > 0.0;
    if (cub) {
      d0 = (k - 1 >= 0) ? (G(k + 1) - G(k - 1)) / (times[k + 1] - times[k - 1]) : (G(k + 1) - G(k)) / (times[k + 1] - times[k]);
      d1 = (k + 2 < N) ? (G(k + 2) - G(k)) / (times[k + 2] - times[k]) : (G(k + 1) - G(k)) / (times[k + 1] - times[k]);
    }
    int accept_left = 0;
    if (fabs(gk) < tol_on_surface) {
      if (direction == 0)
        accept_left = 1;
      else if (direction == 1)
        accept_left = (gk1 >= 0.0) || (k - 1 >= 0 && G(k - 1) <= 0.0);
      else
        accept_left = (gk1 <= 0.0) || (k - 1 >= 0 && G(k - 1) >= 0.0);
      if (accept_left) stop = emit(&E, t0, states + 6 * k);
    }
    for (int mm = 0; mm < r + 1 && !stop; ++mm) {
      const double s_lo = mm * step, s_hi = (mm + 1) * step;
      if (s_hi > 1.0 + 1e-15) break;
      if (accept_left && mm == 0) continue;
      double g_lo, g_hi;
      if (cub) {
        g_lo = herm_s(s_lo, gk, gk1, d0, d1, dt);
        g_hi = herm_s(s_hi, gk, gk1, d0, d1, dt);
      } else {
        g_lo = (1.0 - s_lo) * gk + s_lo * gk1;
        g_hi = (1.0 - s_hi) * gk + s_hi * gk1;
      }
      int crosses;
      if (direction == 0)
        crosses = (g_lo * g_hi <= 0.0) && (g_lo != g_hi);
      else if (direction == 1)
        crosses = (g_lo < 0.0) && (g_hi >= 0.0);
      else
        crosses = (g_lo > 0.0) && (g_hi <= 0.0);
      if (!crosses) continue;
      double s_star;
      if (g_lo == g_hi) {
        s_star = 0.5 * (s_lo + s_hi);
      } else {
        double a = g_lo / (g_lo - g_hi);
        a = (a > 0.0) ? a : 0.0;
        a = (1.0 < a) ? 1.0 : a;
        s_star = s_lo + a * (s_hi - s_lo);
      }
      if (cub) {
        for (int it = 0; it < newton_max_iter; ++it) {
          const double f = herm_s(s_star, gk, gk1, d0, d1, dt);
          const double df = herm_d(s_star, gk, gk1, d0, d1, dt);
          if (df == 0.0) break;
          s_star -= f / df;
          if (s_star < s_lo) { s_star = s_lo; break; }
          if (s_star > s_hi) { s_star = s_hi; break; }
        }
      }
      const double th = (1.0 - s_star) * t0 + s_star * t1;
      double x[6];
      if (cub && k - 1 >= 0 && k + 2 < N) {
        const double s = s_star;
        const double h00 = (1.0 + 2.0 * s) * sq_py(1.0 - s);
        const double h10 = s * sq_py(1.0 - s);
        const double h01 = sq_py(s) * (3.0 - 2.0 * s);
        const double h11 = sq_py(s) * (s - 1.0);
        for (int c = 0; c < 6; ++c) {
          const double dxdt0 = (states[6 * (k + 1) + c] - states[6 * (k - 1) + c]) / (times[k + 1] - times[k - 1]);
          const double dxdt1 = (states[6 * (k + 2) + c] - states[6 * k + c]) / (times[k + 2] - times[k]);
          x[c] = ((h00 * states[6 * k + c] + (h10 * dxdt0) * dt) + h01 * states[6 * (k + 1) + c]) + (h11 * dxdt1) * dt;
        }
      } else {
        for (int c = 0; c < 6; ++c) x[c] = states[6 * k + c] + s_star * (states[6 * (k + 1) + c] - states[6 * k + c]);
      }
      stop = emit(&E, th, x);
    }
  }
#undef G
  *n_stored = E.stored;
  return E.found;
}
