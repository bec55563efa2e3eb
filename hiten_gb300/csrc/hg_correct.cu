// Batched single-shooting correction of halo orbits: a native host driver
// over the propagation kernels (corrector/backends/newton.py:39-143,
// corrector/operators.py:408-452, types/services/orbits.py:851-948,
// corrector/backends/base.py:187-245, corrector/stepping/armijo.py:58-164).
//
// Controls (x0, vy0); residual (vx, vz) at the first y = 0 crossing in the
// half-period window; Jacobian from the STM at that crossing minus the
// quadratic term; step from a 2x2 solve (Tikhonov 1e-12 above the condition
// threshold), capped and line-searched (Armijo) per orbit.  All orbits still
// iterating share each propagation launch.  Host arithmetic follows the
// reference's numpy expressions operation by operation (the library's host
// code is compiled without floating-point contraction and calls C `pow` for
// the reference's scalar `**`); the 2x2 solve reproduces LAPACK's partially
// pivoted elimination as numpy on x86-64 runs it.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "hg_internal.h"
#include "hitengpu.h"

namespace {

// A view into the handle's corrector buffers (Shooter::arena).
struct DevBuf {
  void* p = nullptr;
  double* d() const { return (double*)p; }
  int* i() const { return (int*)p; }
};

struct Shooter {
  hg_handle* h;
  double mu;
  hg_newton_opts o;
  cudaStream_t s;
  int cap;
  // event leg (6-dim), STM leg (42-dim)
  DevBuf y6, ye6, te, ht, hy, nh, na, nr, st, y42, ye42, te42, tm, smp, na42, nr42, st42;
  void* arena = nullptr;  // the handle's corrector buffers, carved into the views above
  std::vector<double> hbuf;
  std::vector<int> ibuf;

  // Byte sizes of the views for `cap` orbits, in carving order; returns the
  // total (256-byte aligned parts).  With `carve` the views are set from
  // `base`.
  size_t layout(char* base, bool carve) {
    const size_t n = (size_t)cap;
    struct Part {
      DevBuf* b;
      size_t bytes;
    } parts[] = {{&y6, 6 * n * 8},   {&ye6, 6 * n * 8},   {&te, n * 8},      {&ht, n * 8},     {&hy, 6 * n * 8},
                 {&nh, n * 4},       {&na, n * 4},        {&nr, n * 4},      {&st, n * 4},     {&y42, 42 * n * 8},
                 {&ye42, 42 * n * 8}, {&te42, n * 8},     {&tm, n * 8},      {&smp, 42 * n * 8}, {&na42, n * 4},
                 {&nr42, n * 4},     {&st42, n * 4}};
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t off = 0;
    for (const Part& q : parts) {
      if (carve) q.b->p = base + off;
      off += up(q.bytes ? q.bytes : 8);
    }
    return off;
  }

  // Buffers from the handle (no allocation once hg_reserve_correct covered
  // `cap` orbits).
  int init() {
    const size_t total = layout(nullptr, false);
    const int rc = hg_internal::correct_buffers(h, (long long)total, &arena);
    if (rc != HG_OK) return rc;
    layout((char*)arena, true);
    return HG_OK;
  }

  // First y = 0 crossing of every state x (M x 6, row-major): t_event = 1e-12 +
  // t_rel, the state there, found (poincare/singlehit/backend.py:164-280).
  int events(const std::vector<double>& x, int M, std::vector<double>& t_event, std::vector<double>& x_ev,
             std::vector<char>& found) {
    hbuf.assign((size_t)6 * M, 0.0);
    for (int i = 0; i < M; ++i)
      for (int c = 0; c < 6; ++c) hbuf[(size_t)c * M + i] = x[(size_t)i * 6 + c];
    if (cudaMemcpyAsync(y6.p, hbuf.data(), hbuf.size() * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return HG_ERR_CUDA;
    const double span = fmax(0.0, M_PI - 1e-12);
    hg_dop853_opts op{o.event_rtol, o.event_atol, INFINITY, 10.0 * 2.220446049250313e-16, 100000, 1, 0, 6};
    hg_event ev{1, 0.0, 0, 1, 1e-12, 1e-12};
    int rc = hg_propagate_dop853(h, mu, 6, M, y6.d(), M, nullptr, nullptr, 0.0, span, &op, &ev, 0, 0, nullptr,
                                 ye6.d(), te.d(), ht.d(), hy.d(), nh.i(), na.i(), nr.i(), st.i(), s);
    if (rc != HG_OK) return rc;
    std::vector<double> hit_t(M), hit_y((size_t)6 * M);
    std::vector<int> n(M);
    if (cudaMemcpyAsync(hit_t.data(), ht.p, (size_t)M * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(hit_y.data(), hy.p, (size_t)6 * M * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(n.data(), nh.p, (size_t)M * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return HG_ERR_CUDA;
    t_event.resize(M);
    x_ev.resize((size_t)M * 6);
    found.resize(M);
    for (int i = 0; i < M; ++i) {
      const double tr = hit_t[i];
      t_event[i] = 1e-12 + tr;
      for (int c = 0; c < 6; ++c) x_ev[(size_t)i * 6 + c] = hit_y[(size_t)c * M + i];
      found[i] = n[i] > 0 && tr < span && tr >= 0.0;
    }
    return HG_OK;
  }

  // Phi(t_event) of every state (dynamics/rtbp.py:258-340, last dense sample).
  int stm(const std::vector<double>& x, int M, const std::vector<double>& t_event, std::vector<double>& Phi) {
    hbuf.assign((size_t)42 * M, 0.0);
    for (int i = 0; i < M; ++i) {
      for (int k = 0; k < 6; ++k) hbuf[(size_t)(7 * k) * M + i] = 1.0;
      for (int c = 0; c < 6; ++c) hbuf[(size_t)(36 + c) * M + i] = x[(size_t)i * 6 + c];
    }
    if (cudaMemcpyAsync(y42.p, hbuf.data(), hbuf.size() * 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(tm.p, t_event.data(), (size_t)M * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return HG_ERR_CUDA;
    hg_dop853_opts op{o.stm_rtol, o.stm_atol, 1e4, 10.0 * 2.220446049250313e-16, 100000, 1, 36, 42};
    int rc = hg_propagate_dop853(h, mu, 42, M, y42.d(), M, nullptr, tm.d(), 0.0, 0.0, &op, nullptr, o.steps, 1,
                                 smp.d(), ye42.d(), te42.d(), nullptr, nullptr, nullptr, na42.i(), nr42.i(), st42.i(),
                                 s);
    if (rc != HG_OK) return rc;
    hbuf.resize((size_t)36 * M);
    if (cudaMemcpyAsync(hbuf.data(), smp.p, (size_t)36 * M * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return HG_ERR_CUDA;
    Phi.resize((size_t)36 * M);
    for (int i = 0; i < M; ++i)
      for (int c = 0; c < 36; ++c) Phi[(size_t)i * 36 + c] = hbuf[(size_t)c * M + i];
    return HG_OK;
  }
};

// types/services/orbits.py:917-948 for one orbit (numpy scalar arithmetic).
void quadratic_term(const double* xe, const double* Phi, double mu, double out[4]) {
  const double x = xe[0], y = xe[1], z = xe[2];
  double vy = xe[4];
  const double mu2 = 1 - mu;
  const double rho_1 = 1 / pow((pow(x + mu, 2) + pow(y, 2)) + pow(z, 2), 1.5);
  const double rho_2 = 1 / pow((pow(x - mu2, 2) + pow(y, 2)) + pow(z, 2), 1.5);
  const double omega_x = (-((mu2 * (x + mu)) * rho_1) - ((mu * (x - mu2)) * rho_2)) + x;
  const double DDx = 2 * vy + omega_x;
  const double DDz = -((mu2 * z) * rho_1) - ((mu * z) * rho_2);
  if (fabs(vy) < 1e-9) vy = vy != 0 ? (vy > 0 ? 1e-9 : -1e-9) : 1e-9;
  const double p0 = Phi[6 * 1 + 0], p4 = Phi[6 * 1 + 4];
  out[0] = DDx * p0 / vy;
  out[1] = DDx * p4 / vy;
  out[2] = DDz * p0 / vy;
  out[3] = DDz * p4 / vy;
}

// 2-norm condition number of a 2x2 matrix from its singular values; used
// only against the regularisation threshold.
double cond2(const double J[4]) {
  const double a = J[0], b = J[1], c = J[2], d = J[3];
  if (!(isfinite(a) && isfinite(b) && isfinite(c) && isfinite(d))) return NAN;
  const double S = ((a * a + b * b) + c * c) + d * d;
  const double D = fabs(a * d - b * c);
  if (D == 0.0) return INFINITY;
  const double disc = sqrt(fmax(S * S - 4.0 * D * D, 0.0));
  const double smax2 = 0.5 * (S + disc);
  const double smin2 = D * D / smax2;
  return sqrt(smax2 / smin2);
}

// numpy.linalg.solve for 2x2 (LAPACK dgesv: partial pivoting, reciprocal
// scaling of the pivot column, fused updates where the x86-64 kernels fuse).
bool solve2(const double J[4], const double b[2], double x[2]) {
  double a00 = J[0], a01 = J[1], a10 = J[2], a11 = J[3], b0 = b[0], b1 = b[1];
  if (fabs(a10) > fabs(a00)) {
    std::swap(a00, a10);
    std::swap(a01, a11);
    std::swap(b0, b1);
  }
  if (a00 == 0.0) return false;
  const double inv00 = 1.0 / a00;
  const double l = a10 * inv00;
  const double u11 = a11 - l * a01;
  if (u11 == 0.0) return false;
  const double y1 = fma(-l, b0, b1);
  const double x1 = y1 / u11;
  const double t = fma(-a01, x1, b0);
  x[0] = t / a00;
  x[1] = x1;
  return true;
}

}  // namespace

extern "C" {

void hg_host_pow(long long n, const double* x, double e, double* out) {
  if (n <= 0 || !x || !out) return;
  for (long long i = 0; i < n; ++i) out[i] = pow(x[i], e);
}

void hg_newton_opts_default(hg_newton_opts* o) {
  if (!o) return;
  o->tol = 1e-12;
  o->max_attempts = 50;
  o->max_delta = 1e-2;
  o->alpha_reduction = 0.5;
  o->min_alpha = 1e-4;
  o->armijo_c = 0.1;
  o->cond_threshold = 1e8;
  o->event_rtol = o->event_atol = 1e-12;
  o->stm_rtol = o->stm_atol = 1e-12;
  o->steps = 500;
}

int hg_reserve_correct(hg_handle* h, int max_orbits) {
  if (!h) return HG_ERR_ARGS;
  if (max_orbits < 0) return hg_internal::fail_msg(h, HG_ERR_ARGS, "hg_reserve_correct: max_orbits < 0");
  hg_newton_opts o;
  hg_newton_opts_default(&o);
  Shooter sh{h, 0.0, o, nullptr, max_orbits};
  int rc = sh.init();
  if (rc != HG_OK) return rc;
  // the half-period legs refine one crossing per orbit
  return hg_internal::reserve_refine(h, max_orbits, 6, 1);
}

int hg_correct_halo(hg_handle* h, double mu, int N, double* x, long long ld, double* half_period, int* iterations,
                    double* residual, int* status, const hg_newton_opts* opts, void* stream) {
  if (!h || N < 0 || (N > 0 && (!x || !half_period || !iterations || !residual || !status)) || ld < N)
    return HG_ERR_ARGS;
  if (N == 0) return HG_OK;
  hg_newton_opts o;
  hg_newton_opts_default(&o);
  if (opts) o = *opts;
  if (o.max_attempts < 1 || !(o.tol > 0) || o.steps < 2) return HG_ERR_ARGS;
  cudaStream_t s = (cudaStream_t)stream;
  Shooter sh{h, mu, o, s, N};
  {
    const int rc0 = sh.init();
    if (rc0 != HG_OK) return rc0;
  }
  // inputs: SoA [6][ld] on the device
  std::vector<double> soa((size_t)6 * N), base((size_t)N * 6);
  for (int c = 0; c < 6; ++c)
    if (cudaMemcpyAsync(soa.data() + (size_t)c * N, x + (size_t)c * ld, (size_t)N * 8, cudaMemcpyDeviceToHost, s) !=
        cudaSuccess)
      return HG_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return HG_ERR_CUDA;
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < 6; ++c) base[(size_t)i * 6 + c] = soa[(size_t)c * N + i];
  std::vector<double> params((size_t)N * 2);
  for (int i = 0; i < N; ++i) {
    params[2 * i] = base[(size_t)i * 6 + 0];
    params[2 * i + 1] = base[(size_t)i * 6 + 4];
  }
  std::vector<int> st_out(N, -1), it_out(N, 0);
  std::vector<double> rn_out(N, NAN), tev_out(N, NAN);
  auto full = [&](const double* p, const std::vector<int>& rows, std::vector<double>& xf) {
    xf.resize(rows.size() * 6);
    for (size_t k = 0; k < rows.size(); ++k) {
      memcpy(&xf[k * 6], &base[(size_t)rows[k] * 6], 6 * 8);
      xf[k * 6 + 0] = p[2 * k];
      xf[k * 6 + 4] = p[2 * k + 1];
    }
  };
  // residual of the controls p of `rows`: r (vx, vz), its inf-norm, t_event, x_event, found
  struct Res {
    std::vector<double> r, rn, tev, xev;
    std::vector<char> found;
  };
  auto residual_of = [&](const std::vector<double>& p, const std::vector<int>& rows, Res& R) -> int {
    std::vector<double> xf;
    full(p.data(), rows, xf);
    const int M = (int)rows.size();
    int rc = sh.events(xf, M, R.tev, R.xev, R.found);
    if (rc != HG_OK) return rc;
    R.r.resize((size_t)M * 2);
    R.rn.resize(M);
    for (int k = 0; k < M; ++k) {
      const double r0 = R.xev[(size_t)k * 6 + 3] - 0.0, r1 = R.xev[(size_t)k * 6 + 5] - 0.0;
      R.r[2 * k] = r0;
      R.r[2 * k + 1] = r1;
      R.rn[k] = fmax(fabs(r0), fabs(r1));
    }
    return HG_OK;
  };

  // trajectories an event leg takes at its per-step latency floor (six lanes
  // per trajectory, four warps per SM: 4 x SMs x 5), at most N
  // (the buffers' capacity)
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                 cudaSuccess || sms < 1)
    sms = 1;
  const int spec_traj = std::max(1, std::min(N, 20 * sms));
  constexpr int kMaxSpec = 8;
  std::vector<int> active(N);
  for (int i = 0; i < N; ++i) active[i] = i;
  Res cur;
  int rc = residual_of(params, active, cur);
  if (rc != HG_OK) return rc;
  {  // orbits without a crossing
    std::vector<int> a2;
    Res c2;
    for (size_t k = 0; k < active.size(); ++k) {
      if (!cur.found[k]) {
        st_out[active[k]] = HG_EVENT_NOT_FOUND;
        continue;
      }
      a2.push_back(active[k]);
      c2.r.push_back(cur.r[2 * k]);
      c2.r.push_back(cur.r[2 * k + 1]);
      c2.rn.push_back(cur.rn[k]);
      c2.tev.push_back(cur.tev[k]);
      c2.xev.insert(c2.xev.end(), cur.xev.begin() + 6 * k, cur.xev.begin() + 6 * k + 6);
    }
    active.swap(a2);
    cur = c2;
  }
  bool exhausted = true;
  for (int k = 0; k < o.max_attempts; ++k) {
    // converged orbits leave
    {
      std::vector<int> a2;
      Res c2;
      for (size_t q = 0; q < active.size(); ++q) {
        const int i = active[q];
        if (cur.rn[q] < o.tol) {
          st_out[i] = HG_OK;
          it_out[i] = k;
          rn_out[i] = cur.rn[q];
          tev_out[i] = cur.tev[q];
          continue;
        }
        a2.push_back(i);
        c2.r.push_back(cur.r[2 * q]);
        c2.r.push_back(cur.r[2 * q + 1]);
        c2.rn.push_back(cur.rn[q]);
        c2.tev.push_back(cur.tev[q]);
        c2.xev.insert(c2.xev.end(), cur.xev.begin() + 6 * q, cur.xev.begin() + 6 * q + 6);
      }
      active.swap(a2);
      cur = c2;
    }
    const int M = (int)active.size();
    if (M == 0) {
      exhausted = false;
      break;
    }
    std::vector<double> pa((size_t)M * 2), xf, Phi;
    for (int q = 0; q < M; ++q) {
      pa[2 * q] = params[2 * active[q]];
      pa[2 * q + 1] = params[2 * active[q] + 1];
    }
    full(pa.data(), active, xf);
    rc = sh.stm(xf, M, cur.tev, Phi);
    if (rc != HG_OK) return rc;
    // Newton step per orbit
    std::vector<double> delta((size_t)M * 2);
    for (int q = 0; q < M; ++q) {
      const double* P = &Phi[(size_t)q * 36];
      double quad[4];
      quadratic_term(&cur.xev[(size_t)q * 6], P, mu, quad);
      double J[4] = {P[6 * 3 + 0] - quad[0], P[6 * 3 + 4] - quad[1], P[6 * 5 + 0] - quad[2], P[6 * 5 + 4] - quad[3]};
      const double cnd = cond2(J);
      if (isnan(cnd) || cnd > o.cond_threshold) {
        J[0] = J[0] + 1e-12;
        J[3] = J[3] + 1e-12;
      }
      const double b[2] = {-cur.r[2 * q], -cur.r[2 * q + 1]};
      double d[2] = {NAN, NAN};
      solve2(J, b, d);
      if (!std::isinf(o.max_delta)) {
        const double dn = fmax(fabs(d[0]), fabs(d[1]));
        if (dn > o.max_delta) {
          d[0] = d[0] * (o.max_delta / dn);
          d[1] = d[1] * (o.max_delta / dn);
        }
      }
      delta[2 * q] = d[0];
      delta[2 * q + 1] = d[1];
    }
    // Armijo line search, batched over the orbits still searching
    std::vector<double> alpha(M, 1.0), best_p = pa, best_n = cur.rn, best_a(M, 0.0), best_r = cur.r,
                                       best_t = cur.tev, best_x = cur.xev;
    std::vector<double> new_p = pa, new_n = cur.rn, new_r = cur.r, new_t = cur.tev, new_x = cur.xev;
    std::vector<char> pending(M, 1), failed(M, 0);
    for (;;) {
      std::vector<int> idx;
      for (int q = 0; q < M; ++q)
        if (pending[q]) idx.push_back(q);
      if (idx.empty()) break;
      // Each round evaluates the next S step fractions alpha, alpha r, ...,
      // alpha r^(S-1) of every pending orbit in one propagation: the event
      // legs of up to spec_traj trajectories run at their per-step latency
      // floor, so the extra trials come almost free, and the decisions below
      // consume them in the sequential order (each trial is the same
      // computation whenever it runs): the results are those of one trial per
      // round, in fewer rounds.
      const int P = (int)idx.size();
      const int S = std::max(1, std::min(kMaxSpec, spec_traj / P));
      std::vector<int> rows((size_t)P * S);
      std::vector<double> trial((size_t)P * S * 2), ta((size_t)P * S);
      for (int u = 0; u < P; ++u) {
        const int q = idx[u];
        double a = alpha[q];
        for (int j = 0; j < S; ++j) {
          const size_t v = (size_t)u * S + j;
          rows[v] = active[q];
          ta[v] = a;
          trial[2 * v] = pa[2 * q] + a * delta[2 * q];
          trial[2 * v + 1] = pa[2 * q + 1] + a * delta[2 * q + 1];
          a *= o.alpha_reduction;
        }
      }
      Res T;
      rc = residual_of(trial, rows, T);
      if (rc != HG_OK) return rc;
      for (int u = 0; u < P; ++u) {
        const int q = idx[u];
        for (int j = 0; j < S && pending[q]; ++j) {
          const size_t v = (size_t)u * S + j;
          const bool ft = T.found[v];
          if (ft && T.rn[v] <= (1.0 - o.armijo_c * alpha[q]) * cur.rn[q]) {
            new_p[2 * q] = trial[2 * v];
            new_p[2 * q + 1] = trial[2 * v + 1];
            new_n[q] = T.rn[v];
            new_r[2 * q] = T.r[2 * v];
            new_r[2 * q + 1] = T.r[2 * v + 1];
            new_t[q] = T.tev[v];
            memcpy(&new_x[(size_t)q * 6], &T.xev[v * 6], 6 * 8);
            pending[q] = 0;
            break;
          }
          if (ft && T.rn[v] < best_n[q]) {
            best_p[2 * q] = trial[2 * v];
            best_p[2 * q + 1] = trial[2 * v + 1];
            best_n[q] = T.rn[v];
            best_a[q] = alpha[q];
            best_r[2 * q] = T.r[2 * v];
            best_r[2 * q + 1] = T.r[2 * v + 1];
            best_t[q] = T.tev[v];
            memcpy(&best_x[(size_t)q * 6], &T.xev[v * 6], 6 * 8);
          }
          alpha[q] *= o.alpha_reduction;
          if (alpha[q] < o.min_alpha) {
            pending[q] = 0;
            if (best_a[q] > 0) {
              new_p[2 * q] = best_p[2 * q];
              new_p[2 * q + 1] = best_p[2 * q + 1];
              new_n[q] = best_n[q];
              new_r[2 * q] = best_r[2 * q];
              new_r[2 * q + 1] = best_r[2 * q + 1];
              new_t[q] = best_t[q];
              memcpy(&new_x[(size_t)q * 6], &best_x[(size_t)q * 6], 6 * 8);
            } else {
              failed[q] = 1;
            }
          }
        }
      }
    }
    std::vector<int> a2;
    Res c2;
    for (int q = 0; q < M; ++q) {
      const int i = active[q];
      if (failed[q]) {
        st_out[i] = HG_LINE_SEARCH_FAILED;
        it_out[i] = k;
        continue;
      }
      params[2 * i] = new_p[2 * q];
      params[2 * i + 1] = new_p[2 * q + 1];
      a2.push_back(i);
      c2.r.push_back(new_r[2 * q]);
      c2.r.push_back(new_r[2 * q + 1]);
      c2.rn.push_back(new_n[q]);
      c2.tev.push_back(new_t[q]);
      c2.xev.insert(c2.xev.end(), new_x.begin() + 6 * q, new_x.begin() + 6 * q + 6);
    }
    active.swap(a2);
    cur = c2;
  }
  if (exhausted) {  // newton.py:130-143: final residual check
    for (size_t q = 0; q < active.size(); ++q) {
      const int i = active[q];
      st_out[i] = cur.rn[q] < o.tol ? HG_OK : HG_NEWTON_DIVERGED;
      it_out[i] = o.max_attempts;
      rn_out[i] = cur.rn[q];
      tev_out[i] = cur.tev[q];
    }
  }
  for (int i = 0; i < N; ++i) {
    base[(size_t)i * 6 + 0] = params[2 * i];
    base[(size_t)i * 6 + 4] = params[2 * i + 1];
    for (int c = 0; c < 6; ++c) soa[(size_t)c * N + i] = base[(size_t)i * 6 + c];
  }
  for (int c = 0; c < 6; ++c)
    if (cudaMemcpyAsync(x + (size_t)c * ld, soa.data() + (size_t)c * N, (size_t)N * 8, cudaMemcpyHostToDevice, s) !=
        cudaSuccess)
      return HG_ERR_CUDA;
  if (cudaMemcpyAsync(half_period, tev_out.data(), (size_t)N * 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(residual, rn_out.data(), (size_t)N * 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(iterations, it_out.data(), (size_t)N * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(status, st_out.data(), (size_t)N * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return HG_ERR_CUDA;
  return HG_OK;
}

}  // extern "C"
