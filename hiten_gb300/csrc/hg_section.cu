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
// same-signed numbers), nor under cubic interpolation while the end values
// clear the Hermite bounds below, so it is skipped without changing any
// result; the scans of the remaining segments are shared by the warp.
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

// Per-lane segment context shared during a cooperative scan.
struct SegCtx {
  double gk, gk1, d0, d1, dt;
  bool cub;
  bool skip0;  // the on-surface left end was accepted: sub-interval 0 is not scanned
};

// Value of g at sub-interval point q (s = q * step) of a segment: the cubic
// Hermite or the linear interpolant, as the reference evaluates it.
__device__ __forceinline__ double seg_point(const SegCtx& c, double s) {
  return c.cub ? hermite_scalar(s, c.gk, c.gk1, c.d0, c.d1, c.dt) : (1.0 - s) * c.gk + s * c.gk1;
}

__device__ __forceinline__ bool sub_crosses(double g_lo, double g_hi, int direction) {
  if (direction == 0) return (g_lo * g_hi <= 0.0) && (g_lo != g_hi);
  if (direction == 1) return (g_lo < 0.0) && (g_hi >= 0.0);
  return (g_lo > 0.0) && (g_hi <= 0.0);
}

// Warp-cooperative detection: the 32 lanes (one trajectory each) walk their
// segments in lock step.  Each lane decides whether its segment can hold a
// crossing (the exact skip tests above); the sub-interval scan of every
// candidate segment is then shared by the whole warp (lane L evaluates the
// sub-intervals 32 c + L, the same expressions on the same operands as the
// sequential scan, so the same values), and every lane refines its own
// crossings in sub-interval order -- Newton and interpolation run across
// lanes instead of one lane at a time.  Results, their order and the
// de-duplication are those of the per-trajectory loop.
__global__ void __launch_bounds__(128) section_kernel(SecParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = i < p.N;
  const int ii = valid ? i : 0;
  Emitter em(p, ii);
  const int N = p.m;
  const int r = p.segment_refine;
  const double step = 1.0 / (double)(r + 1);
  const bool dir_any = p.direction == 0;
  // sub-intervals the reference scans: mm = 0 .. n_sub - 1 (it stops at the
  // first whose upper end exceeds 1 + 1e-15)
  int n_sub = 0;
  while (n_sub <= r && !((double)(n_sub + 1) * step > 1.0 + 1e-15)) ++n_sub;
  const int n_chunks = (n_sub + 31) / 32;
  double g_prev = 0.0;
  double gk = valid && N > 0 ? smp(p, 0, p.axis, ii) - p.offset : 0.0;
  double tk = valid && N > 0 ? tim(p, 0, ii) : 0.0;
  for (int k = 0; k + 1 < N; ++k) {
    const bool live = valid && !em.full;
    if (!__any_sync(0xFFFFFFFFu, live)) break;
    SegCtx c{gk, 0.0, 0.0, 0.0, 0.0, false, false};
    double tk1 = tk;
    bool cand = false;
    if (live) {
      const double gk1 = smp(p, k + 1, p.axis, ii) - p.offset;
      tk1 = tim(p, k + 1, ii);
      const double dt = tk1 - tk;
      c.gk1 = gk1;
      c.dt = dt;
      const bool near = fabs(gk) < p.tol_on_surface;
      const bool same_sign = (gk > 0.0 && gk1 > 0.0) || (gk < 0.0 && gk1 < 0.0);
      // Segments with an end value this small are always scanned.  Without a
      // direction the reference tests g_lo * g_hi <= 0, and that product
      // underflows to zero (a reported crossing) once both factors fall below
      // about 2^-537; 2^-490 keeps every sub-interval value of a skipped
      // segment (linear: at least the smaller end; cubic: above the skip
      // margin 2^-46 (|g0| + |g1| + ...) >= 2^-535) far from that range.
      // With a direction the tests compare g itself with zero, and 1e-280
      // only keeps (1 - s) g away from underflow.
      const double tiny_end = dir_any ? 0x1p-490 : 1e-280;
      const bool tiny = fabs(gk) < tiny_end || fabs(gk1) < tiny_end;
      cand = true;
      if (!near && same_sign && !tiny && !p.cubic) cand = false;
      if (cand) {
        c.cub = p.cubic && dt > 0.0;
        if (c.cub) {
          if (k - 1 >= 0)
            c.d0 = (gk1 - g_prev) / (tk1 - tim(p, k - 1, ii));
          else
            c.d0 = (gk1 - gk) / (tk1 - tk);
          if (k + 2 < N)
            c.d1 = ((smp(p, k + 2, p.axis, ii) - p.offset) - gk) / (tim(p, k + 2, ii) - tk);
          else
            c.d1 = (gk1 - gk) / (tk1 - tk);
        }
        // Cubic segments that cannot cross.  On [0, 1] the Hermite cubic with
        // end values g0, g1 and end slopes m0 = d0 dt, m1 = d1 dt is the
        // Bezier curve with control values g0, g0 + m0/3, g1 - m1/3, g1 and
        // lies in their convex hull; it also satisfies g(s) = g0 H00 + g1 H01
        // + m0 H10 + m1 H11 with H00, H01 >= 0, H00 + H01 = 1, |H10|, |H11|
        // <= 4/27.  When either bound keeps it on the side of the
        // (same-signed) end values by more than 2^-46 (|g0| + |g1| + |m0| +
        // |m1|) -- far above the rounding of any evaluated point (a few
        // ulps) -- no sub-interval value changes sign, and skipping the scan
        // changes no result.
        if (c.cub && !near && same_sign && !tiny) {
          const double m0 = c.d0 * dt, m1 = c.d1 * dt;
          const double am0 = fabs(m0), am1 = fabs(m1);
          const double margin = 0x1p-46 * ((fabs(gk) + fabs(gk1)) + (am0 + am1));
          const double sg = gk > 0.0 ? 1.0 : -1.0;
          const double b1 = sg * (gk + m0 / 3.0), b2 = sg * (gk1 - m1 / 3.0);
          const bool hull = b1 > margin && b2 > margin && fabs(gk) > margin && fabs(gk1) > margin;
          const double lo = fmin(fabs(gk), fabs(gk1));
          const bool basis = lo > (4.0 / 27.0) * (am0 + am1) * (1.0 + 1e-12) + margin;
          if (hull || basis) cand = false;
        }
      }
      if (cand && near) {
        bool accept_left;
        if (dir_any)
          accept_left = true;
        else if (p.direction == 1)
          accept_left = (gk1 >= 0.0) || (k - 1 >= 0 && g_prev <= 0.0);
        else
          accept_left = (gk1 <= 0.0) || (k - 1 >= 0 && g_prev >= 0.0);
        if (accept_left) {
          double x[6];
#pragma unroll
          for (int cc = 0; cc < 6; ++cc) x[cc] = smp(p, k, cc, ii);
          em.offer(tk, x);
          c.skip0 = true;
        }
      }
      if (em.full) cand = false;
    }
    const unsigned cmask = __ballot_sync(0xFFFFFFFFu, cand);
    for (int ch = 0; ch < n_chunks && cmask; ++ch) {
      // scan chunk ch of every candidate segment with the whole warp
      unsigned my_bits = 0;
      for (unsigned rest = cmask; rest; rest &= rest - 1) {
        const int j = __ffs(rest) - 1;
        SegCtx cj;
        cj.gk = __shfl_sync(0xFFFFFFFFu, c.gk, j);
        cj.gk1 = __shfl_sync(0xFFFFFFFFu, c.gk1, j);
        cj.d0 = __shfl_sync(0xFFFFFFFFu, c.d0, j);
        cj.d1 = __shfl_sync(0xFFFFFFFFu, c.d1, j);
        cj.dt = __shfl_sync(0xFFFFFFFFu, c.dt, j);
        cj.cub = __shfl_sync(0xFFFFFFFFu, (int)c.cub, j) != 0;
        cj.skip0 = __shfl_sync(0xFFFFFFFFu, (int)c.skip0, j) != 0;
        const int mm = 32 * ch + lane;
        bool x = false;
        if (mm < n_sub && !(cj.skip0 && mm == 0)) {
          const double g_lo = seg_point(cj, (double)mm * step);
          const double g_hi = seg_point(cj, (double)(mm + 1) * step);
          x = sub_crosses(g_lo, g_hi, p.direction);
        }
        const unsigned bits = __ballot_sync(0xFFFFFFFFu, x);
        if (lane == j) my_bits = bits;
      }
      // every lane refines its own crossings of this chunk, in order
      while (my_bits && !em.full) {
        const int mm = 32 * ch + __ffs(my_bits) - 1;
        my_bits &= my_bits - 1;
        const double s_lo = (double)mm * step;
        const double s_hi = (double)(mm + 1) * step;
        const double g_lo = seg_point(c, s_lo);
        const double g_hi = seg_point(c, s_hi);
        double s_star;
        if (g_lo == g_hi) {
          s_star = 0.5 * (s_lo + s_hi);
        } else {
          double a = g_lo / (g_lo - g_hi);
          a = fmin(1.0, fmax(0.0, a));
          s_star = s_lo + a * (s_hi - s_lo);
        }
        if (c.cub) {
          for (int it = 0; it < p.newton_max_iter; ++it) {
            const double f = hermite_scalar(s_star, c.gk, c.gk1, c.d0, c.d1, c.dt);
            const double df = hermite_der(s_star, c.gk, c.gk1, c.d0, c.d1, c.dt);
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
        const double dt = c.dt;
        double x[6];
        if (c.cub && k - 1 >= 0 && k + 2 < N) {
          const double tm1 = tim(p, k - 1, ii), tp2 = tim(p, k + 2, ii);
          const double s = s_star;
          const double om = 1.0 - s;
          const double h00 = (1.0 + 2.0 * s) * (om * om);
          const double h10 = s * (om * om);
          const double h01 = (s * s) * (3.0 - 2.0 * s);
          const double h11 = (s * s) * (s - 1.0);
#pragma unroll
          for (int cc = 0; cc < 6; ++cc) {
            const double dxdt0 = (smp(p, k + 1, cc, ii) - smp(p, k - 1, cc, ii)) / (tk1 - tm1);
            const double dxdt1 = (smp(p, k + 2, cc, ii) - smp(p, k, cc, ii)) / (tp2 - tk);
            x[cc] = ((h00 * smp(p, k, cc, ii) + (h10 * dxdt0) * dt) + h01 * smp(p, k + 1, cc, ii)) + (h11 * dxdt1) * dt;
          }
        } else {
#pragma unroll
          for (int cc = 0; cc < 6; ++cc) {
            const double a0 = smp(p, k, cc, ii);
            x[cc] = a0 + s_star * (smp(p, k + 1, cc, ii) - a0);
          }
        }
        em.offer(th, x);
      }
    }
    if (live) {
      g_prev = gk;
      gk = c.gk1;
      tk = tk1;
    }
  }
  if (valid) {
    p.n_hits[i] = em.stored;
    if (p.n_found) p.n_found[i] = em.found;
  }
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
