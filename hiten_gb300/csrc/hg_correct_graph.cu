// Batched single-shooting halo correction run on the device as one CUDA
// graph (hg_correct_halo_graph): the Newton iterations of every orbit and
// their Armijo line searches are two nested conditional WHILE nodes, the
// propagation legs are the library's DOP853 kernels in list mode (they read
// the number of live trajectories from device memory), and the Newton
// algebra, line-search decisions and list compaction are small kernels in
// between.  The host enqueues one graph launch per call; nothing is read back
// until the caller synchronizes.
//
// The iteration follows the host drivers (hg_correct.cu, corrector.py), which
// restate corrector/backends/newton.py:39-143, corrector/operators.py:408-452,
// types/services/orbits.py:851-948, corrector/backends/base.py:187-245 and
// corrector/stepping/armijo.py:58-164: the residual (vx, vz) at the first
// y = 0 crossing of the half-period window (poincare/singlehit/backend.py:
// 164-280: 1e-12 alignment, window [0, pi - 1e-12], undirected system), the
// Jacobian Phi[[3,5],[0,4]] minus the quadratic term, Tikhonov 1e-12 above
// the condition threshold, a 2x2 solve with LAPACK's pivoting, the step cap,
// and the Armijo search with the next S step fractions of every pending orbit
// evaluated in one propagation and consumed in the sequential order.  The one
// arithmetic difference from the host drivers: the quadratic term's powers
// are correctly rounded (x * x, hg_pow15) where the host calls the C
// library's pow.
//
// Termination does not depend on the logic being right: the outer loop runs
// at most max_attempts times and the inner at most kMaxRounds times per
// Newton iteration (the body kernels count unconditionally), and every
// propagation is bounded by its step budget.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <mutex>
#include <new>

#include "hg_internal.h"
#include "hg_kernels.cuh"
#include "hg_pair.cuh"
#include "hitengpu.h"

namespace {

constexpr int kMaxRounds = 64;          // line-search rounds per Newton iteration (alpha halves to 1e-4 in 14)
constexpr int kMaxAttemptsCap = 1000;   // largest max_attempts accepted
constexpr int kSegSteps = 1 << 20;      // one list-mode launch runs every trajectory to its end
constexpr int kBlockCtl = 1024;         // threads of the single-block control kernels
constexpr double kSpan = 3.141592653589793 - 1e-12;  // max(0, pi - 1e-12): the window past the alignment

// Per-orbit and per-slot device state, carved from the caller's workspace.
struct Ws {
  int N, cap;
  // per orbit (index i)
  double *base;                 // [6][N] initial guesses
  double *p0, *p1;              // controls x0, vy0
  double *r0, *r1, *rn, *tev;   // current residual, its inf-norm, crossing time
  double *xev;                  // [6][N] crossing state
  double *d0, *d1;              // Newton step
  double *x0p0, *x0p1;          // controls at the start of the line search
  double *alpha;
  double *bp0, *bp1, *bn, *ba, *br0, *br1, *bt, *bx;  // best trial ([6][N] for bx)
  double *np0, *np1, *nn, *nr0, *nr1, *nt, *nx;       // accepted step ([6][N] for nx)
  double *rnorm, *tevo;        // outputs
  int *st, *it, *active, *pending, *failed;
  int *act;                    // [N] active orbits (ordered)
  // per trial slot (index v < cap)
  int *rows;                   // orbit of the slot
  double *tp0, *tp1;           // trial controls
  int *tfound;
  double *tr0, *tr1, *trn, *ttev, *txev;  // residual of the slot ([6][cap] for txev)
  // event leg (6-dim)
  double *ey0, *eyend, *etend, *ehitt, *ehity;
  int *enh, *ena, *enr, *est;
  // STM leg (42-dim)
  double *sy0, *syend, *stend, *stmax, *ssmp;
  int *sna, *snr, *sst;
  // list mode
  int *iota, *dummy_out;
  double *wh, *wep, *wpp;
  int *wq;
  char* refine;
  // scalars
  int* sc;  // [0] trial slots, [1] STM slots, [2] k, [3] rounds, [4] active orbits M, [5] trials per
           // pending orbit S, [6] spec_traj, [7] list-mode output count (unused)
};

long long up(long long x) { return (x + 255) & ~255LL; }

long long refine_bytes(int N) {
  const long long cap = N;  // one crossing per trajectory
  return 256 + 2 * up(cap * 4) + up((15LL * 6 + 3) * cap * 8);
}

long long layout(int N, char* b, Ws* w) {
  long long off = 0;
  const long long nd = up(8LL * N), ni = up(4LL * N);
  auto D = [&](double** p, int k) {
    if (w) *p = (double*)(b + off);
    off += k * nd;
  };
  auto I = [&](int** p, int k) {
    if (w) *p = (int*)(b + off);
    off += k * ni;
  };
  Ws dummy;
  Ws* x = w ? w : &dummy;
  D(&x->base, 6); D(&x->p0, 1); D(&x->p1, 1); D(&x->r0, 1); D(&x->r1, 1); D(&x->rn, 1); D(&x->tev, 1);
  D(&x->xev, 6); D(&x->d0, 1); D(&x->d1, 1); D(&x->x0p0, 1); D(&x->x0p1, 1); D(&x->alpha, 1);
  D(&x->bp0, 1); D(&x->bp1, 1); D(&x->bn, 1); D(&x->ba, 1); D(&x->br0, 1); D(&x->br1, 1); D(&x->bt, 1);
  D(&x->bx, 6); D(&x->np0, 1); D(&x->np1, 1); D(&x->nn, 1); D(&x->nr0, 1); D(&x->nr1, 1); D(&x->nt, 1);
  D(&x->nx, 6); D(&x->rnorm, 1); D(&x->tevo, 1);
  I(&x->st, 1); I(&x->it, 1); I(&x->active, 1); I(&x->pending, 1); I(&x->failed, 1); I(&x->act, 1);
  I(&x->rows, 1); D(&x->tp0, 1); D(&x->tp1, 1); I(&x->tfound, 1); D(&x->tr0, 1); D(&x->tr1, 1); D(&x->trn, 1);
  D(&x->ttev, 1); D(&x->txev, 6);
  D(&x->ey0, 6); D(&x->eyend, 6); D(&x->etend, 1); D(&x->ehitt, 1); D(&x->ehity, 6);
  I(&x->enh, 1); I(&x->ena, 1); I(&x->enr, 1); I(&x->est, 1);
  D(&x->sy0, 42); D(&x->syend, 42); D(&x->stend, 1); D(&x->stmax, 1); D(&x->ssmp, 42);
  I(&x->sna, 1); I(&x->snr, 1); I(&x->sst, 1);
  I(&x->iota, 1); I(&x->dummy_out, 1); D(&x->wh, 1); D(&x->wep, 1); D(&x->wpp, 1); I(&x->wq, 1);
  if (w) w->refine = b + off;
  off += refine_bytes(N);
  if (w) w->sc = (int*)(b + off);
  off += 256;
  if (w) {
    w->N = N;
    w->cap = N;
  }
  return off;
}

// Block-wide ordered compaction step: for flag f of thread t in the current
// chunk, returns its position among the flagged threads of the chunk and
// adds the chunk's count to *total (all threads see the same *total after).
__device__ int block_excl_scan(int f, int* sm_warp, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const unsigned bal = __ballot_sync(0xFFFFFFFFu, f);
  const int before_in_warp = __popc(bal & ((1u << lane) - 1u));
  if (lane == 0) sm_warp[w] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int q = 0; q < nw; ++q) {
      const int c = sm_warp[q];
      sm_warp[q] = s;
      s += c;
    }
    sm_warp[nw] = s;
  }
  __syncthreads();
  const int pos = *total + sm_warp[w] + before_in_warp;
  const int chunk = sm_warp[nw];
  __syncthreads();
  if (threadIdx.x == 0) *total += chunk;
  __syncthreads();
  return pos;
}

// Trial states for the event leg: slot v holds orbit rows[v]'s guess with
// the trial controls; status -2 (not started) so the list-mode launch starts
// it from y0; the refinement record count is cleared.
__global__ void gc_trial_states(Ws w) {
  const int n = w.sc[0];
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int i = w.rows[v];
#pragma unroll
    for (int c = 0; c < 6; ++c) w.ey0[(long long)c * w.cap + v] = w.base[(long long)c * w.N + i];
    w.ey0[v] = w.tp0[v];
    w.ey0[4LL * w.cap + v] = w.tp1[v];
    w.est[v] = -2;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // refine_count lives at the start of the refinement area
    *(int*)w.refine = 0;
  }
}

// Residual of every trial slot from the event leg (singlehit window test).
__global__ void gc_trial_residual(Ws w) {
  const int n = w.sc[0];
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const double t_rel = w.ehitt[v];
    const bool found = w.enh[v] > 0 && t_rel < kSpan && t_rel >= 0.0;
    double xe[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      xe[c] = w.ehity[(long long)c * w.cap + v];
      w.txev[(long long)c * w.cap + v] = xe[c];
    }
    const double a = xe[3] - 0.0, b = xe[5] - 0.0;
    w.tfound[v] = found ? 1 : 0;
    w.tr0[v] = a;
    w.tr1[v] = b;
    w.trn[v] = fmax(fabs(a), fabs(b));
    w.ttev[v] = 1e-12 + t_rel;
  }
}

// Set-up: controls from the guesses, every orbit running, one trial slot per
// orbit for the first residual.
__global__ void gc_init(Ws w, int spec_traj) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.N; i += gridDim.x * blockDim.x) {
    w.p0[i] = w.base[i];
    w.p1[i] = w.base[4LL * w.N + i];
    w.st[i] = -1;
    w.it[i] = 0;
    w.rnorm[i] = NAN;
    w.tevo[i] = NAN;
    w.active[i] = 1;
    w.rows[i] = i;
    w.tp0[i] = w.p0[i];
    w.tp1[i] = w.p1[i];
    w.iota[i] = i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.sc[0] = w.N;
    w.sc[1] = 0;
    w.sc[2] = 0;
    w.sc[3] = 0;
    w.sc[4] = 0;
    w.sc[5] = 0;
    w.sc[6] = spec_traj;
  }
}

__device__ void take_trial(const Ws& w, int v, double* r0, double* r1, double* rn, double* tev, double* xev,
                           int i) {
  r0[i] = w.tr0[v];
  r1[i] = w.tr1[v];
  rn[i] = w.trn[v];
  tev[i] = w.ttev[v];
#pragma unroll
  for (int c = 0; c < 6; ++c) xev[(long long)c * w.N + i] = w.txev[(long long)c * w.cap + v];
}

// First residual: orbits without a crossing leave with HG_EVENT_NOT_FOUND.
__global__ void gc_first_residual(Ws w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.N; i += gridDim.x * blockDim.x) {
    if (!w.tfound[i]) {
      w.st[i] = HG_EVENT_NOT_FOUND;
      w.active[i] = 0;
      continue;
    }
    take_trial(w, i, w.r0, w.r1, w.rn, w.tev, w.xev, i);
  }
}

// Top of Newton iteration k: converged orbits leave; the STM leg's states for
// the others (Phi = I, the current state; up to the crossing time).
__global__ void __launch_bounds__(kBlockCtl) gc_converge(Ws w, double tol) {
  __shared__ int sm[34];
  __shared__ int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  const int k = w.sc[2];
  for (int base = 0; base < w.N; base += blockDim.x) {
    const int i = base + threadIdx.x;
    int keep = 0;
    if (i < w.N && w.active[i]) {
      if (w.rn[i] < tol) {
        w.st[i] = HG_OK;
        w.it[i] = k;
        w.rnorm[i] = w.rn[i];
        w.tevo[i] = w.tev[i];
        w.active[i] = 0;
      } else {
        keep = 1;
      }
    }
    const int q = block_excl_scan(keep, sm, &total);
    if (keep) w.act[q] = i;
  }
  __syncthreads();
  const int M = total;
  for (int q = threadIdx.x; q < M; q += blockDim.x) {
    const int i = w.act[q];
    for (int c = 0; c < 36; ++c) w.sy0[(long long)c * w.cap + q] = (c % 7 == 0) ? 1.0 : 0.0;
    for (int c = 0; c < 6; ++c) w.sy0[(long long)(36 + c) * w.cap + q] = w.base[(long long)c * w.N + i];
    w.sy0[36LL * w.cap + q] = w.p0[i];
    w.sy0[40LL * w.cap + q] = w.p1[i];
    w.stmax[q] = w.tev[i];
    w.sst[q] = -2;
  }
  if (threadIdx.x == 0) {
    w.sc[4] = M;
    w.sc[1] = M;
  }
}

// types/services/orbits.py:917-948 for one orbit, powers correctly rounded.
__device__ void quadratic_term(const double xe[6], double p0, double p4, double mu, double out[4]) {
  const double x = xe[0], y = xe[1], z = xe[2];
  double vy = xe[4];
  const double mu2 = 1 - mu;
  const double a = x + mu, b = x - mu2;
  const double rho_1 = 1 / hg_pow15((a * a + y * y) + z * z);
  const double rho_2 = 1 / hg_pow15((b * b + y * y) + z * z);
  const double omega_x = (-((mu2 * (x + mu)) * rho_1) - ((mu * (x - mu2)) * rho_2)) + x;
  const double DDx = 2 * vy + omega_x;
  const double DDz = -((mu2 * z) * rho_1) - ((mu * z) * rho_2);
  if (fabs(vy) < 1e-9) vy = vy != 0 ? (vy > 0 ? 1e-9 : -1e-9) : 1e-9;
  out[0] = DDx * p0 / vy;
  out[1] = DDx * p4 / vy;
  out[2] = DDz * p0 / vy;
  out[3] = DDz * p4 / vy;
}

// 2-norm condition number of a 2x2 matrix (its singular values).
__device__ double cond2(const double J[4]) {
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

// numpy.linalg.solve for 2x2 as LAPACK dgesv rounds it (partial pivoting,
// fused updates as the x86-64 kernels fuse).
__device__ bool solve2(const double J[4], const double b[2], double x[2]) {
  double a00 = J[0], a01 = J[1], a10 = J[2], a11 = J[3], b0 = b[0], b1 = b[1];
  if (fabs(a10) > fabs(a00)) {
    double t = a00; a00 = a10; a10 = t;
    t = a01; a01 = a11; a11 = t;
    t = b0; b0 = b1; b1 = t;
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

// Newton step of every active orbit from its STM at the crossing, and the
// line search's starting state; the inner loop runs while some orbit does.
__global__ void gc_newton(Ws w, double mu, double cond_threshold, double max_delta,
                          cudaGraphConditionalHandle inner) {
  const int M = w.sc[4];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < M; q += gridDim.x * blockDim.x) {
    const int i = w.act[q];
    double P[36];
#pragma unroll
    for (int c = 0; c < 36; ++c) P[c] = w.ssmp[(long long)c * w.cap + q];
    double xe[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) xe[c] = w.xev[(long long)c * w.N + i];
    double quad[4];
    quadratic_term(xe, P[6 * 1 + 0], P[6 * 1 + 4], mu, quad);
    double J[4] = {P[6 * 3 + 0] - quad[0], P[6 * 3 + 4] - quad[1], P[6 * 5 + 0] - quad[2], P[6 * 5 + 4] - quad[3]};
    const double cnd = cond2(J);
    if (isnan(cnd) || cnd > cond_threshold) {
      J[0] = J[0] + 1e-12;
      J[3] = J[3] + 1e-12;
    }
    const double b[2] = {-w.r0[i], -w.r1[i]};
    double d[2] = {NAN, NAN};
    solve2(J, b, d);
    if (!isinf(max_delta)) {
      const double dn = fmax(fabs(d[0]), fabs(d[1]));
      if (dn > max_delta) {
        d[0] = d[0] * (max_delta / dn);
        d[1] = d[1] * (max_delta / dn);
      }
    }
    w.d0[i] = d[0];
    w.d1[i] = d[1];
    w.x0p0[i] = w.p0[i];
    w.x0p1[i] = w.p1[i];
    w.alpha[i] = 1.0;
    w.pending[i] = 1;
    w.failed[i] = 0;
    w.bp0[i] = w.np0[i] = w.p0[i];
    w.bp1[i] = w.np1[i] = w.p1[i];
    w.bn[i] = w.nn[i] = w.rn[i];
    w.ba[i] = 0.0;
    w.br0[i] = w.nr0[i] = w.r0[i];
    w.br1[i] = w.nr1[i] = w.r1[i];
    w.bt[i] = w.nt[i] = w.tev[i];
#pragma unroll
    for (int c = 0; c < 6; ++c) w.bx[(long long)c * w.N + i] = w.nx[(long long)c * w.N + i] = xe[c];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.sc[3] = 0;
    cudaGraphSetConditional(inner, M > 0 ? 1u : 0u);
  }
}

// One line-search round's trials: the next S step fractions alpha r^j of
// every pending orbit (repeated products, as the sequential search forms
// them), S = max(1, min(8, spec_traj / P)).
__global__ void __launch_bounds__(kBlockCtl) gc_trials(Ws w, double alpha_reduction) {
  __shared__ int sm[34];
  __shared__ int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  const int M = w.sc[4];
  // pending orbits in active order: their list goes to dummy_out
  for (int base = 0; base < M; base += blockDim.x) {
    const int q = base + threadIdx.x;
    const int i = q < M ? w.act[q] : 0;
    const int f = (q < M && w.pending[i]) ? 1 : 0;
    const int u = block_excl_scan(f, sm, &total);
    if (f) w.dummy_out[u] = i;
  }
  __syncthreads();
  const int P = total;
  const int spec = w.sc[6];
  const int S = P > 0 ? max(1, min(8, spec / P)) : 1;
  for (int u = threadIdx.x; u < P; u += blockDim.x) {
    const int i = w.dummy_out[u];
    double a = w.alpha[i];
    for (int j = 0; j < S; ++j) {
      const int v = u * S + j;
      w.rows[v] = i;
      w.tp0[v] = w.x0p0[i] + a * w.d0[i];
      w.tp1[v] = w.x0p1[i] + a * w.d1[i];
      a *= alpha_reduction;
    }
  }
  if (threadIdx.x == 0) {
    w.sc[0] = P * S;
    w.sc[5] = S;  // trials per pending orbit in this round
  }
}

// The round's decisions in the sequential order of the line search
// (stepping/armijo.py:58-164); the loop continues while an orbit is pending
// and fewer than kMaxRounds rounds ran.
__global__ void __launch_bounds__(kBlockCtl) gc_decide(Ws w, double armijo_c, double alpha_reduction,
                                                       double min_alpha, cudaGraphConditionalHandle inner) {
  const int S = w.sc[5];
  const int P = S > 0 ? w.sc[0] / S : 0;
  for (int u = threadIdx.x; u < P; u += blockDim.x) {
    const int i = w.dummy_out[u];
    for (int j = 0; j < S && w.pending[i]; ++j) {
      const int v = u * S + j;
      const bool ft = w.tfound[v] != 0;
      const double nj = w.trn[v];
      if (ft && nj <= (1.0 - armijo_c * w.alpha[i]) * w.rn[i]) {
        w.np0[i] = w.tp0[v];
        w.np1[i] = w.tp1[v];
        take_trial(w, v, w.nr0, w.nr1, w.nn, w.nt, w.nx, i);
        w.pending[i] = 0;
        break;
      }
      if (ft && nj < w.bn[i]) {
        w.bp0[i] = w.tp0[v];
        w.bp1[i] = w.tp1[v];
        w.ba[i] = w.alpha[i];
        take_trial(w, v, w.br0, w.br1, w.bn, w.bt, w.bx, i);
      }
      w.alpha[i] *= alpha_reduction;
      if (w.alpha[i] < min_alpha) {
        w.pending[i] = 0;
        if (w.ba[i] > 0) {
          w.np0[i] = w.bp0[i];
          w.np1[i] = w.bp1[i];
          w.nn[i] = w.bn[i];
          w.nr0[i] = w.br0[i];
          w.nr1[i] = w.br1[i];
          w.nt[i] = w.bt[i];
#pragma unroll
          for (int c = 0; c < 6; ++c) w.nx[(long long)c * w.N + i] = w.bx[(long long)c * w.N + i];
        } else {
          w.failed[i] = 1;
        }
      }
    }
  }
  __syncthreads();
  const int M = w.sc[4];
  int any = 0;
  for (int q = threadIdx.x; q < M; q += blockDim.x) any |= w.pending[w.act[q]];
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) {
    const int rounds = w.sc[3] + 1;
    w.sc[3] = rounds;
    if (any && rounds >= kMaxRounds) {
      // cannot happen (alpha falls below min_alpha first); end the search as a failure
      for (int q = 0; q < M; ++q) {
        const int i = w.act[q];
        if (w.pending[i]) {
          w.pending[i] = 0;
          w.failed[i] = 1;
        }
      }
      any = 0;
    }
    cudaGraphSetConditional(inner, any ? 1u : 0u);
  }
}

// End of Newton iteration k: failed searches leave with
// HG_LINE_SEARCH_FAILED, the others take their step; after the last
// iteration the remaining orbits get the final residual check
// (newton.py:130-143).  The outer loop continues while orbits are active
// and k < max_attempts.
__global__ void __launch_bounds__(kBlockCtl) gc_apply(Ws w, double tol, int max_attempts,
                                                      cudaGraphConditionalHandle outer) {
  const int M = w.sc[4];
  const int k = w.sc[2];
  int any = 0;
  for (int q = threadIdx.x; q < M; q += blockDim.x) {
    const int i = w.act[q];
    if (w.failed[i]) {
      w.st[i] = HG_LINE_SEARCH_FAILED;
      w.it[i] = k;
      w.active[i] = 0;
      continue;
    }
    w.p0[i] = w.np0[i];
    w.p1[i] = w.np1[i];
    w.r0[i] = w.nr0[i];
    w.r1[i] = w.nr1[i];
    w.rn[i] = w.nn[i];
    w.tev[i] = w.nt[i];
    for (int c = 0; c < 6; ++c) w.xev[(long long)c * w.N + i] = w.nx[(long long)c * w.N + i];
    if (k + 1 >= max_attempts) {
      w.st[i] = w.rn[i] < tol ? HG_OK : HG_NEWTON_DIVERGED;
      w.it[i] = max_attempts;
      w.rnorm[i] = w.rn[i];
      w.tevo[i] = w.tev[i];
      w.active[i] = 0;
    } else {
      any = 1;
    }
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) {
    w.sc[2] = k + 1;
    cudaGraphSetConditional(outer, (any && k + 1 < max_attempts) ? 1u : 0u);
  }
}

// Caller's outputs: corrected states, half periods, residuals, iterations, status.
__global__ void gc_output(Ws w, double* x, long long ld, double* half_period, int* iterations, double* residual,
                          int* status) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.N; i += gridDim.x * blockDim.x) {
    for (int c = 0; c < 6; ++c) x[(long long)c * ld + i] = w.base[(long long)c * w.N + i];
    x[i] = w.p0[i];
    x[4 * ld + i] = w.p1[i];
    half_period[i] = w.tevo[i];
    residual[i] = w.rnorm[i];
    iterations[i] = w.it[i];
    status[i] = w.st[i];
  }
}

__global__ void gc_load(Ws w, const double* x, long long ld) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.N; i += gridDim.x * blockDim.x)
    for (int c = 0; c < 6; ++c) w.base[(long long)c * w.N + i] = x[(long long)c * ld + i];
}

// ---------------------------------------------------------------------------
// Launch helpers (captured into the graph)

struct Dev {
  int sms = 0;
};

template <class K>
int resident_blocks(K kern, int block, int sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return per_sm * sms;
}

// The event leg on trial slots [0, sc[0]): DOP853 in list mode with the
// undirected y = 0 event, then the lock-step refinement of the crossings.
template <int G>
void event_leg(const Ws& w, double mu, const hg_newton_opts& o, int sms, cudaStream_t s, int* launches) {
  const int ctl = (w.cap + 255) / 256;
  gc_trial_states<<<ctl < 1 ? 1 : ctl, 256, 0, s>>>(w);
  hg::DopParams p;
  memset(&p, 0, sizeof(p));
  p.N = w.cap;
  p.mu = mu;
  p.dir.neg_lo = 0;
  p.dir.neg_hi = 0;
  p.y0 = w.ey0;
  p.ld = w.cap;
  p.t0 = 0.0;
  p.tmax = kSpan;
  p.rtol = o.event_rtol;
  p.atol = o.event_atol;
  p.max_step = INFINITY;
  p.min_step = 10.0 * 2.220446049250313e-16;
  p.max_steps = 100000;
  p.ev_index = 1;
  p.ev_offset = 0.0;
  p.ev_dir = 0;
  p.max_hits = 1;
  p.xtol = 1e-12;
  p.gtol = 1e-12;
  p.y_end = w.eyend;
  p.t_end = w.etend;
  p.hit_t = w.ehitt;
  p.hit_y = w.ehity;
  p.n_hits = w.enh;
  p.n_accept = w.ena;
  p.n_reject = w.enr;
  p.status = w.est;
  p.seg = 1;
  p.seg_steps = kSegSteps;
  p.active_in = w.iota;
  p.n_in = w.sc + 0;
  p.active_out = w.wq;
  p.n_out = w.sc + 7;
  p.ws_h = w.wh;
  p.ws_err_prev = w.wep;
  p.ws_prev_pow = w.wpp;
  p.ws_q = w.wq;
  // the refinement pool (one crossing per trajectory)
  const long long capr = w.cap;
  p.refine_count = (int*)w.refine;
  p.refine_list = (int*)(w.refine + 256);
  p.refine_hit = (int*)(w.refine + 256 + up(capr * 4));
  p.rec = (double*)(w.refine + 256 + 2 * up(capr * 4));
  p.rec_ld = capr;
  const int tpb = hg::Layout<G>::TPW;
  const int need = (w.cap + tpb - 1) / tpb;
  const int cap_blocks = resident_blocks(hg::dop853_kernel<G, false>, 32, sms);
  const int grid = need < cap_blocks ? need : cap_blocks;
  p.stride = grid * tpb;
  hg::dop853_kernel<G, false><<<grid, 32, 0, s>>>(p);
  // refinement of the saved crossings (records [0, refine_count))
  const int rneed = (int)((capr + 31) / 32);
  const int rcap = resident_blocks(hg::refine_kernel<1>, 32, sms);
  const int rgrid = rneed < rcap ? rneed : rcap;
  hg::DopParams q = p;
  q.stride = rgrid * 32;
  hg::refine_kernel<1><<<rgrid, 32, 0, s>>>(q);
  gc_trial_residual<<<ctl < 1 ? 1 : ctl, 256, 0, s>>>(w);
  *launches += 4;
}

// The STM leg on slots [0, sc[1]): 42-dim DOP853 in list mode to each
// orbit's crossing time, the last of o.steps dense samples (rtbp.py:258-340).
template <int G>
void stm_leg(const Ws& w, double mu, const hg_newton_opts& o, int sms, cudaStream_t s, int* launches) {
  hg::DopParams p;
  memset(&p, 0, sizeof(p));
  p.N = w.cap;
  p.mu = mu;
  p.dir.neg_lo = 0;
  p.dir.neg_hi = 0;
  p.y0 = w.sy0;
  p.ld = w.cap;
  p.t0 = 0.0;
  p.tmax_arr = w.stmax;
  p.rtol = o.stm_rtol;
  p.atol = o.stm_atol;
  p.max_step = 1e4;
  p.min_step = 10.0 * 2.220446049250313e-16;
  p.max_steps = 100000;
  p.ev_index = -1;
  p.m = o.steps;
  p.dense_last = 1;
  p.y_out = w.ssmp;
  p.y_end = w.syend;
  p.t_end = w.stend;
  p.n_accept = w.sna;
  p.n_reject = w.snr;
  p.status = w.sst;
  p.seg = 1;
  p.seg_steps = kSegSteps;
  p.active_in = w.iota;
  p.n_in = w.sc + 1;
  p.active_out = w.wq;
  p.n_out = w.sc + 7;
  p.ws_h = w.wh;
  p.ws_err_prev = w.wep;
  p.ws_prev_pow = w.wpp;
  p.ws_q = w.wq;
  if constexpr (G == 12 || G == 18) {
    // the paired (12) and three-warp (18) layouts: five trajectories per
    // block, the live count read from n_in (their list is the identity)
    const int grid = (w.cap + hg::kPairTraj - 1) / hg::kPairTraj;
    if constexpr (G == 18)
      hg::dop853_trio_kernel<<<grid, 96, 0, s>>>(p);
    else
      hg::dop853_pair_kernel<<<grid, 64, 0, s>>>(p);
  } else {
    const int tpb = hg::Layout<G>::TPW;
    const int need = (w.cap + tpb - 1) / tpb;
    const int cap_blocks = resident_blocks(hg::dop853_kernel<G, true>, 32, sms);
    const int grid = need < cap_blocks ? need : cap_blocks;
    p.stride = grid * tpb;
    hg::dop853_kernel<G, true><<<grid, 32, 0, s>>>(p);
  }
  *launches += 1;
}

int lanes_d6(int n, int sms, int tuned) {
  if (tuned == 1 || tuned == 2 || tuned == 6) return tuned;
  const long long smsp = 4LL * sms;
  if ((n + 4LL) / 5 <= smsp) return 6;
  if ((n + 15LL) / 16 <= smsp) return 2;
  return 1;
}

// STM leg layout: the handle's tuning, else the three-warp layout while its
// warps fit about three per SM (3 N / 5 <= 3 x SMs) and the paired warps above
// (the host driver's rule for event-free 42-dim legs).
int lanes_d42(int tuned, int n, int sms) {
  if (tuned == 7 || tuned == 14 || tuned == 12 || tuned == 18) return tuned;
  return 3LL * ((n + hg::kPairTraj - 1) / hg::kPairTraj) <= 3LL * sms ? 18 : 12;
}

void event_leg_any(int g, const Ws& w, double mu, const hg_newton_opts& o, int sms, cudaStream_t s, int* n) {
  if (g == 6)
    event_leg<6>(w, mu, o, sms, s, n);
  else if (g == 2)
    event_leg<2>(w, mu, o, sms, s, n);
  else
    event_leg<1>(w, mu, o, sms, s, n);
}

// Cached instantiated graph of one problem shape.
struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  void* ws = nullptr;
  int N = 0;
  double mu = 0.0;
  hg_newton_opts o;
  int g6 = 0, g42 = 0, kernels = 0;
};

bool same_opts(const hg_newton_opts& a, const hg_newton_opts& b) {
  return a.tol == b.tol && a.max_attempts == b.max_attempts && a.max_delta == b.max_delta &&
         a.alpha_reduction == b.alpha_reduction && a.min_alpha == b.min_alpha && a.armijo_c == b.armijo_c &&
         a.cond_threshold == b.cond_threshold && a.event_rtol == b.event_rtol && a.event_atol == b.event_atol &&
         a.stm_rtol == b.stm_rtol && a.stm_atol == b.stm_atol && a.steps == b.steps;
}

void free_cache(void* p) {
  GraphCache* c = (GraphCache*)p;
  if (!c) return;
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  delete c;
}

// The leaf node of a graph built by one stream capture (a chain).
cudaError_t leaf_of(cudaGraph_t g, cudaGraphNode_t* leaf) {
  size_t n = 0;
  cudaError_t e = cudaGraphGetNodes(g, nullptr, &n);
  if (e != cudaSuccess || n == 0) return e != cudaSuccess ? e : cudaErrorInvalidValue;
  cudaGraphNode_t nodes[64];
  if (n > 64) return cudaErrorInvalidValue;
  e = cudaGraphGetNodes(g, nodes, &n);
  if (e != cudaSuccess) return e;
  for (size_t k = 0; k < n; ++k) {
    size_t nd = 0;
    e = cudaGraphNodeGetDependentNodes(nodes[k], nullptr, nullptr, &nd);
    if (e != cudaSuccess) return e;
    if (nd == 0) {
      *leaf = nodes[k];
      return cudaSuccess;
    }
  }
  return cudaErrorInvalidValue;
}

// Builds the correction graph: set-up and first residual, then
// WHILE(outer) { converge; STM leg; Newton step; WHILE(inner) { trials;
// event leg; decisions }; apply }.
cudaError_t build_graph(const Ws& w, double mu, const hg_newton_opts& o, int g6, int g42, int sms, int spec_traj,
                        cudaStream_t s, cudaGraph_t* out, int* kernels) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  int nk = 0;
  auto fail = [&](cudaError_t err) {
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(s, &junk);
      if (junk && junk != g) cudaGraphDestroy(junk);
    }
    cudaGraphDestroy(g);
    cudaGetLastError();
    return err;
  };
  const int blocks = (w.N + 255) / 256;
  // prologue
  if ((e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return fail(e);
  gc_init<<<blocks, 256, 0, s>>>(w, spec_traj);
  ++nk;
  event_leg_any(g6, w, mu, o, sms, s, &nk);
  gc_first_residual<<<blocks, 256, 0, s>>>(w);
  ++nk;
  if ((e = cudaStreamEndCapture(s, &g)) != cudaSuccess) return fail(e);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  cudaGraphNode_t tail;
  if ((e = leaf_of(g, &tail)) != cudaSuccess) return fail(e);
  // outer loop
  cudaGraphConditionalHandle outer;
  if ((e = cudaGraphConditionalHandleCreate(&outer, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return fail(e);
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = outer;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t outer_node;
  if ((e = cudaGraphAddNode(&outer_node, g, &tail, nullptr, 1, &cp)) != cudaSuccess) return fail(e);
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  cudaGraphConditionalHandle inner;
  if ((e = cudaGraphConditionalHandleCreate(&inner, body, 0, 0)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return fail(e);
  gc_converge<<<1, kBlockCtl, 0, s>>>(w, o.tol);
  if (g42 == 7)
    stm_leg<7>(w, mu, o, sms, s, &nk);
  else if (g42 == 14)
    stm_leg<14>(w, mu, o, sms, s, &nk);
  else if (g42 == 18)
    stm_leg<18>(w, mu, o, sms, s, &nk);
  else
    stm_leg<12>(w, mu, o, sms, s, &nk);
  gc_newton<<<blocks, 256, 0, s>>>(w, mu, o.cond_threshold, o.max_delta, inner);
  nk += 2;
  cudaGraph_t body_g = body;
  if ((e = cudaStreamEndCapture(s, &body_g)) != cudaSuccess) return fail(e);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  cudaGraphNode_t body_tail;
  if ((e = leaf_of(body, &body_tail)) != cudaSuccess) return fail(e);
  cudaGraphNodeParams ip = {};
  ip.type = cudaGraphNodeTypeConditional;
  ip.conditional.handle = inner;
  ip.conditional.type = cudaGraphCondTypeWhile;
  ip.conditional.size = 1;
  cudaGraphNode_t inner_node;
  if ((e = cudaGraphAddNode(&inner_node, body, &body_tail, nullptr, 1, &ip)) != cudaSuccess) return fail(e);
  cudaGraph_t ibody = ip.conditional.phGraph_out[0];
  if ((e = cudaStreamBeginCaptureToGraph(s, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return fail(e);
  gc_trials<<<1, kBlockCtl, 0, s>>>(w, o.alpha_reduction);
  event_leg_any(g6, w, mu, o, sms, s, &nk);
  gc_decide<<<1, kBlockCtl, 0, s>>>(w, o.armijo_c, o.alpha_reduction, o.min_alpha, inner);
  nk += 2;
  cudaGraph_t ibody_g = ibody;
  if ((e = cudaStreamEndCapture(s, &ibody_g)) != cudaSuccess) return fail(e);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  // after the inner loop: apply (depends on the inner conditional node)
  if ((e = cudaStreamBeginCaptureToGraph(s, body, &inner_node, nullptr, 1, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return fail(e);
  gc_apply<<<1, kBlockCtl, 0, s>>>(w, o.tol, o.max_attempts, outer);
  ++nk;
  body_g = body;
  if ((e = cudaStreamEndCapture(s, &body_g)) != cudaSuccess) return fail(e);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  *out = g;
  *kernels = nk;
  return cudaSuccess;
}

}  // namespace

extern "C" {

long long hg_correct_halo_graph_workspace_bytes(int N) {
  if (N < 0) return -1;
  return layout(N > 0 ? N : 1, nullptr, nullptr);
}

int hg_correct_halo_graph(hg_handle* h, double mu, int N, double* x, long long ld, double* half_period,
                          int* iterations, double* residual, int* status, const hg_newton_opts* opts,
                          void* workspace, long long workspace_bytes, void* stream) {
  if (!h || N < 0 || N > (1 << 22) || ld < N) return HG_ERR_ARGS;
  if (N > 0 && (!x || !half_period || !iterations || !residual || !status)) return HG_ERR_ARGS;
  hg_newton_opts o;
  hg_newton_opts_default(&o);
  if (opts) o = *opts;
  if (o.max_attempts < 1 || o.max_attempts > kMaxAttemptsCap || !(o.tol > 0) || o.steps < 2 ||
      !(o.alpha_reduction > 0.0 && o.alpha_reduction < 1.0) || !(o.min_alpha > 0.0))
    return hg_internal::fail_msg(h, HG_ERR_ARGS, "hg_correct_halo_graph: invalid options");
  if (N == 0) return HG_OK;
  if (!workspace || workspace_bytes < layout(N, nullptr, nullptr) || ((uintptr_t)workspace & 255) != 0)
    return hg_internal::fail_msg(h, HG_ERR_ARGS,
                                 "workspace smaller than hg_correct_halo_graph_workspace_bytes(N) or not 256-aligned");
  const int device = hg_internal::device_of(h);
  if (cudaSetDevice(device) != cudaSuccess) return hg_internal::fail_msg(h, HG_ERR_CUDA, "cudaSetDevice");
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1)
    return hg_internal::fail_msg(h, HG_ERR_CUDA, "device attributes");
  cudaStream_t s = (cudaStream_t)stream;
  Ws w;
  layout(N, (char*)workspace, &w);
  const int spec_traj = N < 20 * sms ? N : 20 * sms;
  const int g6 = lanes_d6(N, sms, hg_internal::tuning(h, HG_TUNE_DOP853_LANES_D6));
  const int g42 = lanes_d42(hg_internal::tuning(h, HG_TUNE_LANES_D42), N, sms);
  void** slot = hg_internal::graph_slot(h, free_cache);
  GraphCache* c = (GraphCache*)*slot;
  const bool hit = c && c->ws == workspace && c->N == N && c->mu == mu && same_opts(c->o, o) && c->g6 == g6 &&
                   c->g42 == g42;
  if (!hit) {
    if (c) {
      free_cache(c);
      *slot = nullptr;
    }
    c = new (std::nothrow) GraphCache();
    if (!c) return hg_internal::fail_msg(h, HG_ERR_CUDA, "out of host memory");
    // capture on a private stream: the caller's may be the legacy default
    // stream, which cannot be captured; the graph is launched on the caller's
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
      e = build_graph(w, mu, o, g6, g42, sms, spec_traj, cs, &c->graph, &c->kernels);
      cudaStreamDestroy(cs);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->exec, c->graph, 0);
    if (e != cudaSuccess) {
      free_cache(c);
      cudaGetLastError();
      return hg_internal::fail_msg(h, HG_ERR_CUDA, cudaGetErrorString(e));
    }
    c->ws = workspace;
    c->N = N;
    c->mu = mu;
    c->o = o;
    c->g6 = g6;
    c->g42 = g42;
    *slot = c;
  }
  const int blocks = (N + 255) / 256;
  gc_load<<<blocks, 256, 0, s>>>(w, x, ld);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaGraphLaunch(c->exec, s);
  if (e == cudaSuccess) {
    gc_output<<<blocks, 256, 0, s>>>(w, x, ld, half_period, iterations, residual, status);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return hg_internal::fail_msg(h, HG_ERR_CUDA, cudaGetErrorString(e));
  hg_internal::count_launches(h, 3);
  return HG_OK;
}

}  // extern "C"
