// Section-crossing detection on sampled trajectories (the synodic Poincare
// map), restating poincare/synodic/backend.py:458-659
// (_detect_with_segment_refine) and :382-455 (_order_and_dedup_hits) for an
// axis-aligned plane g = y[axis] - offset (SynodicMapConfig's section_axis /
// section_offset), linear sub-segment interpolation (the reference's
// default, see backend.py:762) or cubic Hermite with Newton refinement.
//
// One thread per trajectory walks its samples in order.  The reference
// scans every segment in (segment_refine + 1) sub-intervals; a segment whose
// end values are both strictly positive or both strictly negative (and not
// within the on-surface tolerance) cannot produce a crossing under linear
// interpolation (every sub-interval value is a convex combination of two
// same-signed numbers), so it is skipped without changing any result.
// Candidates are generated in segment order, which is the reference's
// stable ordering, and deduplicated against the last accepted hit as they
// stream out.  HBM-bound: each sample is read once (coalesced: samples are
// [m][6][ld], consecutive threads read consecutive trajectories).
#include <cuda_runtime.h>
#include <math.h>

#include "hitengpu.h"

namespace {

struct SecParams {
  int N, m;
  const double* samples;  // [m][6][ld]
  long long ld;
  const double* times;    // [m][ld] (times_ld = ld) or [m] shared (times_ld = 0)
  long long times_ld;
  int axis;
  double offset;
  int direction;  // -1, 0 (any), +1
  int pu, pv;     // plane coordinates (projection) indices
  int segment_refine;
  int cubic;
  int newton_max_iter;
  double tol_on_surface, dedup_time_tol, dedup_point_tol;
  int max_hits;
  double* hit_t;  // [max_hits][ld]
  double* hit_y;  // [max_hits][6][ld]
  int* n_hits;    // stored hits
  int* n_found;   // accepted hits, including those beyond max_hits
};

__device__ __forceinline__ double smp(const SecParams& p, int q, int c, int i) {
  return p.samples[((long long)q * 6 + c) * p.ld + i];
}
__device__ __forceinline__ double tim(const SecParams& p, int q, int i) {
  return p.times_ld ? p.times[(long long)q * p.times_ld + i] : p.times[q];
}

// poincare/utils.py:53-147 (_hermite_scalar, _hermite_der: squares as x*x,
// the derivative is dH/ds), left-to-right association as written there.
__device__ __forceinline__ double hermite_scalar(double s, double y0, double y1, double dy0, double dy1, double dt) {
  const double om = 1.0 - s;
  const double h00 = (1.0 + 2.0 * s) * (om * om);
  const double h10 = s * (om * om);
  const double h01 = (s * s) * (3.0 - 2.0 * s);
  const double h11 = (s * s) * (s - 1.0);
  return ((h00 * y0 + (h10 * dy0) * dt) + h01 * y1) + (h11 * dy1) * dt;
}
__device__ __forceinline__ double hermite_der(double s, double y0, double y1, double dy0, double dy1, double dt) {
  const double om = 1.0 - s;
  const double dh00 = ((6.0 * s) * (s - 1.0) + (om * om) * 2.0) - (2.0 * om) * (1.0 + 2.0 * s);
  const double dh10 = om * om + s * (2.0 * (s - 1.0));
  const double dh01 = (6.0 * s) * om - (2.0 * s) * (3.0 - 2.0 * s);
  const double dh11 = (2.0 * s) * (s - 1.0) + s * s;
  return ((dh00 * y0 + (dh10 * dy0) * dt) + dh01 * y1) + (dh11 * dy1) * dt;
}

struct Emitter {
  const SecParams& p;
  int i;
  int stored = 0, found = 0;
  bool have = false;
  double pt = 0.0, pu = 0.0, pvv = 0.0;
  bool full = false;
  __device__ Emitter(const SecParams& pp, int ii) : p(pp), i(ii) {}
  // _order_and_dedup_hits: skip near-duplicates of the last accepted hit
  __device__ void offer(double th, const double (&x)[6]) {
    if (full) return;
    double u = x[0], v = x[0];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      if (c == p.pu) u = x[c];
      if (c == p.pv) v = x[c];
    }
    if (have) {
      if (fabs(th - pt) <= p.dedup_time_tol) return;
      const double du = u - pu, dv = v - pvv;
      if ((du * du + dv * dv) <= (p.dedup_point_tol * p.dedup_point_tol)) return;
    }
    have = true;
    pt = th;
    pu = u;
    pvv = v;
    ++found;
    if (stored < p.max_hits) {
      p.hit_t[(long long)stored * p.ld + i] = th;
#pragma unroll
      for (int c = 0; c < 6; ++c) p.hit_y[((long long)stored * 6 + c) * p.ld + i] = x[c];
      ++stored;
      if (stored >= p.max_hits) full = true;  // max_hits_per_traj cap (backend.py:451-452)
    }
  }
};

__global__ void __launch_bounds__(128) section_kernel(SecParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  Emitter em(p, i);
  const int N = p.m;
  const int r = p.segment_refine;
  const double step = 1.0 / (double)(r + 1);
  const bool dir_any = p.direction == 0;
  double g_prev = 0.0;
  double gk = smp(p, 0, p.axis, i) - p.offset;
  double tk = tim(p, 0, i);
  for (int k = 0; k + 1 < N && !em.full; ++k) {
    const double gk1 = smp(p, k + 1, p.axis, i) - p.offset;
    const double tk1 = tim(p, k + 1, i);
    const double dt = tk1 - tk;
    const bool near = fabs(gk) < p.tol_on_surface;
    const bool same_sign = (gk > 0.0 && gk1 > 0.0) || (gk < 0.0 && gk1 < 0.0);
    const bool tiny = fabs(gk) < 1e-280 || fabs(gk1) < 1e-280;
    if (!near && same_sign && !tiny && !p.cubic) {
      g_prev = gk;
      gk = gk1;
      tk = tk1;
      continue;
    }
    double d0 = 0.0, d1 = 0.0;
    const bool cub = p.cubic && dt > 0.0;
    if (cub) {
      if (k - 1 >= 0)
        d0 = (gk1 - g_prev) / (tk1 - tim(p, k - 1, i));
      else
        d0 = (gk1 - gk) / (tk1 - tk);
      if (k + 2 < N)
        d1 = ((smp(p, k + 2, p.axis, i) - p.offset) - gk) / (tim(p, k + 2, i) - tk);
      else
        d1 = (gk1 - gk) / (tk1 - tk);
    }
    bool accept_left = false;
    if (near) {
      if (dir_any)
        accept_left = true;
      else if (p.direction == 1)
        accept_left = (gk1 >= 0.0) || (k - 1 >= 0 && g_prev <= 0.0);
      else
        accept_left = (gk1 <= 0.0) || (k - 1 >= 0 && g_prev >= 0.0);
      if (accept_left) {
        double x[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) x[c] = smp(p, k, c, i);
        em.offer(tk, x);
      }
    }
    for (int mm = 0; mm <= r && !em.full; ++mm) {
      const double s_lo = (double)mm * step;
      const double s_hi = (double)(mm + 1) * step;
      if (s_hi > 1.0 + 1e-15) break;
      if (accept_left && mm == 0) continue;
      double g_lo, g_hi;
      if (cub) {
        g_lo = hermite_scalar(s_lo, gk, gk1, d0, d1, dt);
        g_hi = hermite_scalar(s_hi, gk, gk1, d0, d1, dt);
      } else {
        g_lo = (1.0 - s_lo) * gk + s_lo * gk1;
        g_hi = (1.0 - s_hi) * gk + s_hi * gk1;
      }
      bool crosses;
      if (dir_any)
        crosses = (g_lo * g_hi <= 0.0) && (g_lo != g_hi);
      else if (p.direction == 1)
        crosses = (g_lo < 0.0) && (g_hi >= 0.0);
      else
        crosses = (g_lo > 0.0) && (g_hi <= 0.0);
      if (!crosses) continue;
      double s_star;
      if (g_lo == g_hi) {
        s_star = 0.5 * (s_lo + s_hi);
      } else {
        double a = g_lo / (g_lo - g_hi);
        a = fmin(1.0, fmax(0.0, a));
        s_star = s_lo + a * (s_hi - s_lo);
      }
      if (cub) {
        for (int it = 0; it < p.newton_max_iter; ++it) {
          const double f = hermite_scalar(s_star, gk, gk1, d0, d1, dt);
          const double df = hermite_der(s_star, gk, gk1, d0, d1, dt);
          if (df == 0.0) break;
          s_star -= f / df;
          if (s_star < s_lo) {
            s_star = s_lo;
            break;
          }
          if (s_star > s_hi) {
            s_star = s_hi;
            break;
          }
        }
      }
      const double th = (1.0 - s_star) * tk + s_star * tk1;
      double x[6];
      if (cub && k - 1 >= 0 && k + 2 < N) {
        const double tm1 = tim(p, k - 1, i), tp2 = tim(p, k + 2, i);
        const double s = s_star;
        const double om = 1.0 - s;
        const double h00 = (1.0 + 2.0 * s) * (om * om);
        const double h10 = s * (om * om);
        const double h01 = (s * s) * (3.0 - 2.0 * s);
        const double h11 = (s * s) * (s - 1.0);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const double dxdt0 = (smp(p, k + 1, c, i) - smp(p, k - 1, c, i)) / (tk1 - tm1);
          const double dxdt1 = (smp(p, k + 2, c, i) - smp(p, k, c, i)) / (tp2 - tk);
          x[c] = ((h00 * smp(p, k, c, i) + (h10 * dxdt0) * dt) + h01 * smp(p, k + 1, c, i)) + (h11 * dxdt1) * dt;
        }
      } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const double a0 = smp(p, k, c, i);
          x[c] = a0 + s_star * (smp(p, k + 1, c, i) - a0);
        }
      }
      em.offer(th, x);
    }
    g_prev = gk;
    gk = gk1;
    tk = tk1;
  }
  p.n_hits[i] = em.stored;
  if (p.n_found) p.n_found[i] = em.found;
}

// Manifold acceptance filters on sampled trajectories
// (types/services/manifold.py:412-432): minimum distances to the primaries
// (np.sqrt((x + mu)**2 + y**2 + z**2), numpy squares being x*x) and the
// maximum relative Jacobi-constant drift of common/energy.py:26-74
// (numba: squares x*x, **0.5 of a positive number = the correctly rounded
// square root).  One thread per trajectory.
__global__ void __launch_bounds__(128) filters_kernel(int N, int m, const double* samples, long long ld, double mu,
                                                       double* min_r1, double* min_r2, double* max_rel_e) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double mu1 = 1.0 - mu, mu2 = mu;
  double C0 = 0.0, absC0 = 0.0, emax = 0.0, m1 = 0.0, m2 = 0.0;
  for (int q = 0; q < m; ++q) {
    const double* s = samples + (long long)q * 6 * ld + i;
    const double x = s[0], y = s[ld], z = s[2 * ld], vx = s[3 * ld], vy = s[4 * ld], vz = s[5 * ld];
    const double a = x + mu, b = (x - 1.0) + mu;
    const double d1 = sqrt((a * a + y * y) + z * z);
    const double d2 = sqrt((b * b + y * y) + z * z);
    m1 = (q == 0 || d1 < m1) ? d1 : m1;
    m2 = (q == 0 || d2 < m2) ? d2 : m2;
    const double e = x + mu2, f = x - mu1;
    const double r1 = sqrt((e * e + y * y) + z * z);
    const double r2 = sqrt((f * f + y * y) + z * z);
    const double C = ((x * x + y * y) + 2.0 * (mu1 / r1 + mu2 / r2)) - ((vx * vx + vy * vy) + vz * vz);
    if (q == 0) {
      C0 = C;
      absC0 = fabs(C0);
    } else {
      const double rel = absC0 > 1e-14 ? fabs(C - C0) / absC0 : fabs(C - C0);
      if (rel > emax) emax = rel;
    }
  }
  min_r1[i] = m1;
  min_r2[i] = m2;
  max_rel_e[i] = emax;
}

}  // namespace

extern "C" int hg_trajectory_filters(int N, int m, const double* samples, long long ld, double mu, double* min_r1,
                                     double* min_r2, double* max_rel_energy, void* stream) {
  if (N < 0 || m < 1 || ld < N) return HG_ERR_ARGS;
  if (N > 0 && (!samples || !min_r1 || !min_r2 || !max_rel_energy)) return HG_ERR_ARGS;
  if (N == 0) return HG_OK;
  const int block = 128;
  filters_kernel<<<(N + block - 1) / block, block, 0, (cudaStream_t)stream>>>(N, m, samples, ld, mu, min_r1, min_r2,
                                                                              max_rel_energy);
  return cudaGetLastError() == cudaSuccess ? HG_OK : HG_ERR_CUDA;
}

extern "C" int hg_section_detect(int N, int m, const double* samples, long long ld, const double* times,
                                 long long times_ld, int axis, double offset, int direction, int plane_u,
                                 int plane_v, int segment_refine, int cubic, int newton_max_iter,
                                 double tol_on_surface, double dedup_time_tol, double dedup_point_tol, int max_hits,
                                 double* hit_t, double* hit_y, int* n_hits, int* n_found, void* stream) {
  if (N < 0 || m < 0 || ld < N || (times_ld != 0 && times_ld < N)) return HG_ERR_ARGS;
  if (axis < 0 || axis > 5 || plane_u < 0 || plane_u > 5 || plane_v < 0 || plane_v > 5) return HG_ERR_ARGS;
  if (direction < -1 || direction > 1 || segment_refine < 1 || max_hits < 1 || newton_max_iter < 0) return HG_ERR_ARGS;
  if (N > 0 && (!samples || !times || !hit_t || !hit_y || !n_hits)) return HG_ERR_ARGS;
  if (N == 0) return HG_OK;
  SecParams p;
  p.N = N;
  p.m = m;
  p.samples = samples;
  p.ld = ld;
  p.times = times;
  p.times_ld = times_ld;
  p.axis = axis;
  p.offset = offset;
  p.direction = direction;
  p.pu = plane_u;
  p.pv = plane_v;
  p.segment_refine = segment_refine;
  p.cubic = cubic ? 1 : 0;
  p.newton_max_iter = newton_max_iter;
  p.tol_on_surface = tol_on_surface;
  p.dedup_time_tol = dedup_time_tol;
  p.dedup_point_tol = dedup_point_tol;
  p.max_hits = max_hits;
  p.hit_t = hit_t;
  p.hit_y = hit_y;
  p.n_hits = n_hits;
  p.n_found = n_found;
  const int block = 128;
  section_kernel<<<(N + block - 1) / block, block, 0, (cudaStream_t)stream>>>(p);
  return cudaGetLastError() == cudaSuccess ? HG_OK : HG_ERR_CUDA;
}
