// Paired-warp layout for the 42-dim variational system: fixed-step RK
// (fixed_rk_pair_kernel) and single-pass DOP853 without an event
// (dop853_pair_kernel).
//
// Why.  On GB300 a warp has one FP64 instruction in flight at a time, for
// 64 cycles whatever the number of active lanes (76 when four warps share the
// SM's FP64 unit), so one warp's step costs (its FP64 instructions) x 64-76
// cycles.  A batch of about a thousand 42-dim trajectories gives only a few
// warps per SM, and its time is the per-warp instruction count of a step.
// The state of a trajectory (6 components, the Hessian of the potential and
// the accelerations) and its STM (36 components, F(x) Phi) are two
// instruction streams; run on two warps of one block they split that count.
//
// Layout.  A trajectory group is five trajectories served by two warps:
//   * the state warp: lane 6t + j (t < 5, j < 6) holds state component 36 + j
//     of trajectory t and does job j of the shared Hessian (hessian_split);
//     lanes 30 and 31 shadow group 4 (they repeat job 0 and write nothing);
//   * the STM warp: lane 6t + c holds column c of Phi (components 6r + c,
//     r = 0..5); lanes 30 and 31 shadow column 5 of trajectory 4.
// At every right-hand-side evaluation the state warp forms the Hessian's
// six entries from its stage state (the off-diagonal ones as the products
// hessian42 takes) and hands them to the STM warp through shared memory: a
// ring of kPairSlots slots with an mbarrier pair per slot, "full" after the state warp wrote
// it, "empty" after the STM warp read it; meanwhile the STM warp forms its
// stage columns.  Every operation and operand is the one the 7-lane layout
// uses (Layout<7>), so the results are bit-identical.
//
// Waits are bounded: a hand-off that has not completed within
// kPairWaitNs of wall time marks the warp broken; it stops waiting and
// arriving, the partner's waits run out in turn, both leave the step loop
// and the group's trajectories report HG_SYNC_TIMEOUT.
#pragma once

#include "hg_kernels.cuh"

namespace hg {

constexpr unsigned long long kPairWaitNs = 2000000000ull;  // 2 s per hand-off
constexpr int kPairTraj = 5;                                // trajectories per warp pair
constexpr unsigned kPairSlots = 4;                          // hand-off ring depth

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  [[maybe_unused]] unsigned long long state;
  asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred P;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, P;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the completion of the phase with the given parity; false when it
// has not completed within limit_ns (or 2^30 polls).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity,
                                          unsigned long long limit_ns = kPairWaitNs) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned it = 1; it < (1u << 30); ++it) {
    if (mbar_test(bar, parity)) return true;
    if ((it & 63u) == 0 && global_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// Self-test of the bounded wait (one block of two warps): warp 0 waits on a
// barrier that nothing arrives at and must give up after limit_ns; then warp
// 1 arrives at a second barrier and warp 0's wait on it must succeed.
// out[0] = 1 if the first wait ran out, out[1] = 1 if the second completed,
// out[2] = elapsed nanoseconds of the first wait.
static __global__ void bounded_wait_selftest_kernel(int* out, unsigned long long limit_ns) {
  __shared__ unsigned long long bars[2];
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 32);
    mbar_init(&bars[1], 32);
  }
  __syncthreads();
  const int w = threadIdx.x >> 5;
  if (w == 0) {
    const unsigned long long t0 = global_ns();
    const bool ok0 = mbar_wait(&bars[0], 0, limit_ns);  // nothing arrives
    const unsigned long long dt = global_ns() - t0;
    const bool ran_out = !__any_sync(0xFFFFFFFFu, ok0);
    const bool ok1 = __all_sync(0xFFFFFFFFu, mbar_wait(&bars[1], 0, limit_ns));
    if (threadIdx.x == 0) {
      out[0] = ran_out ? 1 : 0;
      out[1] = ok1 ? 1 : 0;
      out[2] = (int)(dt > 2000000000ull ? 2000000000ull : dt);
    }
  } else {
    mbar_arrive(&bars[1]);
  }
}

// Shared-memory hand-off of one warp pair.
struct PairLink {
  double H[kPairSlots][kPairTraj][8];  // slot, trajectory, (xx, yy, zz, xy, yz, xz, -, -)
  unsigned long long full[kPairSlots];
  unsigned long long empty[kPairSlots];
  int fin[kPairTraj];     // STM columns finite, per trajectory
  int broken;             // STM warp gave up a wait
};

// Lane placement shared by both warps of a pair.
struct PairLane {
  int t;           // trajectory in the group (0..4)
  int role;        // 0..5; 6 and 7 on the shadow lanes 30, 31
  int base;        // first lane of the trajectory
  unsigned gmask;  // lanes of the trajectory (group 4 includes the shadows)
  __device__ __forceinline__ explicit PairLane(int lane) {
    t = lane < 30 ? lane / 6 : 4;
    role = lane < 30 ? lane % 6 : lane - 24;
    base = 6 * t;
    gmask = t < 4 ? (0x3Fu << base) : 0xFF000000u;
  }
};

// State warp: one state component per lane (NC = 1).
struct PairState {
  static constexpr int D = 42;
  static constexpr int NC = 1;
  static constexpr bool kState = true;
  __device__ __forceinline__ int flag_slot() const { return 42; }  // gather-slot flag entry
  int role, base, t;
  unsigned gmask;
  PairLink* link;
  mutable unsigned seq;  // right-hand-side evaluations so far
  mutable bool broken;
  __device__ __forceinline__ int comp(int) const { return 36 + (role < 6 ? role : 0); }
  __device__ __forceinline__ double from(double v, int r) const { return __shfl_sync(gmask, v, base + r); }
  __device__ __forceinline__ void rhs(const double (&v)[1], double mu, const Dir& dir, double (&dv)[1]) const {
    const double x = from(v[0], 0), y = from(v[0], 1), z = from(v[0], 2);
    const double vx = from(v[0], 3), vy = from(v[0], 4);
    // position lanes: their derivative is the velocity of lane role + 3
    const double u = from(v[0], role < 3 ? role + 3 : 0);
    const Hess H = hessian_split<PairState, false>(*this, role < 6 ? role : 0, x, y, z, vx, vy, mu);
    const unsigned b = seq % kPairSlots, use = seq / kPairSlots;
    if (!broken && use >= 1) {
      // the slot's previous contents must have been read (a warp-uniform outcome)
      const bool ok = mbar_wait(&link->empty[b], (use - 1u) & 1u);
      broken = !__all_sync(0xFFFFFFFFu, ok);
    }
    if (!broken) {
      // the six Hessian entries xx, yy, zz, xy, yz, xz: lanes 3..5 formed
      // the off-diagonal ones as hessian42 does (H.xy holds this lane's)
      const double off = H.xy;
      if (role < 6) link->H[b][t][role] = role == 0 ? H.xx : (role == 1 ? H.yy : (role == 2 ? H.zz : off));
      mbar_arrive(&link->full[b]);
    }
    ++seq;
    const double d = role < 3 ? u : (role == 3 ? H.ax : (role == 4 ? H.ay : H.az));
    const int c = comp(0);
    dv[0] = neg_if(d, c >= dir.neg_lo && c < dir.neg_hi);
  }
};

// STM warp: one column of Phi per lane (NC = 6, rows 0..5).
struct PairStm {
  static constexpr int D = 42;
  static constexpr int NC = 6;
  static constexpr bool kState = false;
  __device__ __forceinline__ int flag_slot() const { return 43; }  // and 44: the whole STM
  int col, t;
  int role, base;  // lane placement (role 0..7, as in the state warp), for group-wide steps
  unsigned gmask;
  PairLink* link;
  mutable unsigned seq;
  mutable bool broken;
  __device__ __forceinline__ int comp(int r) const { return 6 * r + col; }
  __device__ __forceinline__ void rhs(const double (&v)[6], double mu, const Dir& dir, double (&dv)[6]) const {
    (void)mu;
    const unsigned b = seq % kPairSlots;
    double xx = 0.0, yy = 0.0, zz = 0.0, xy = 0.0, xz = 0.0, yz = 0.0;
    if (!broken) {
      const bool ok = mbar_wait(&link->full[b], (seq / kPairSlots) & 1u);
      broken = !__all_sync(0xFFFFFFFFu, ok);
    }
    if (!broken) {
      const double* e = link->H[b][t];
      xx = e[0];
      yy = e[1];
      zz = e[2];
      xy = e[3];
      yz = e[4];
      xz = e[5];
      mbar_arrive(&link->empty[b]);
    }
    ++seq;
    // rows of F(x) @ Phi[:, col] (dynamics/rtbp.py:204-209), as Layout<7>
    dv[0] = v[3];
    dv[1] = v[4];
    dv[2] = v[5];
    dv[3] = ((xx * v[0] + xy * v[1]) + xz * v[2]) + 2.0 * v[4];
    dv[4] = ((xy * v[0] + yy * v[1]) + yz * v[2]) + (-2.0) * v[3];
    dv[5] = (xz * v[0] + yz * v[1]) + zz * v[2];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      const int c = comp(r);
      dv[r] = neg_if(dv[r], c >= dir.neg_lo && c < dir.neg_hi);
    }
  }
};

// Half-column STM warps of the three-warp layout (dop853_trio_kernel): two
// warps share the 36 STM components of five trajectories.  A half-group of
// six lanes holds three columns of one trajectory (columns 3 half .. 3 half +
// 2), each column on a lane pair as in Layout<14>: the even lane rows 0..2,
// the odd lane rows 3..5; warp w holds half-groups 5w .. 5w + 4 (trajectory
// = half-group / 2, half = half-group % 2).  A half-group is a complete
// six-lane group for the step control (coefficients, norms, step-size
// factor), so each trajectory's two halves take the same decisions.
struct PairStmHalf {
  static constexpr int D = 42;
  static constexpr int NC = 3;
  static constexpr bool kState = false;
  int t, half;
  int role, base;  // lane placement within the half-group (6, 7 on the shadow lanes)
  unsigned gmask;
  PairLink* link;
  mutable unsigned seq;
  mutable bool broken;
  __device__ __forceinline__ int flag_slot() const { return 43 + half; }
  __device__ __forceinline__ int comp(int r) const {
    const int r6 = role % 6;
    return 6 * (3 * (r6 & 1) + r) + 3 * half + (r6 >> 1);
  }
  __device__ __forceinline__ void rhs(const double (&v)[3], double mu, const Dir& dir, double (&dv)[3]) const {
    (void)mu;
    const unsigned b = seq % kPairSlots;
    double xx = 0.0, yy = 0.0, zz = 0.0, xy = 0.0, xz = 0.0, yz = 0.0;
    if (!broken) {
      const bool ok = mbar_wait(&link->full[b], (seq / kPairSlots) & 1u);
      broken = !__all_sync(0xFFFFFFFFu, ok);
    }
    if (!broken) {
      const double* e = link->H[b][t];
      xx = e[0];
      yy = e[1];
      zz = e[2];
      xy = e[3];
      yz = e[4];
      xz = e[5];
      mbar_arrive(&link->empty[b]);
    }
    ++seq;
    // the partner lane (lane ^ 1) holds the other rows of the column
    const double q0 = __shfl_xor_sync(gmask, v[0], 1), q1 = __shfl_xor_sync(gmask, v[1], 1),
                 q2 = __shfl_xor_sync(gmask, v[2], 1);
    // rows 3..5 of F(x) Phi[:, c] (dynamics/rtbp.py:204-209), as Layout<14>
    const double r3 = ((xx * q0 + xy * q1) + xz * q2) + 2.0 * v[1];
    const double r4 = ((xy * q0 + yy * q1) + yz * q2) + (-2.0) * v[0];
    const double r5 = (xz * q0 + yz * q1) + zz * q2;
    const bool pos = ((role % 6) & 1) == 0;
    const double d0 = pos ? q0 : r3, d1 = pos ? q1 : r4, d2 = pos ? q2 : r5;
    dv[0] = neg_if(d0, comp(0) >= dir.neg_lo && comp(0) < dir.neg_hi);
    dv[1] = neg_if(d1, comp(1) >= dir.neg_lo && comp(1) < dir.neg_hi);
    dv[2] = neg_if(d2, comp(2) >= dir.neg_lo && comp(2) < dir.neg_hi);
  }
};

// One warp's part of a fixed-step propagation (rk.py:531-588): loads its
// components, steps through the nodes, writes rows 0, out_every, ...
// Returns whether its components stayed finite.
template <int ORDER, class LT>
__device__ __forceinline__ bool pair_fixed_run(const LT& L, const FixedParams& p, int traj, bool writes) {
  constexpr int NC = LT::NC;
  double y[NC];
#pragma unroll
  for (int r = 0; r < NC; ++r) y[r] = p.y0[(long long)L.comp(r) * p.ld_in + traj];
  if (writes) {
#pragma unroll
    for (int r = 0; r < NC; ++r) p.out[(long long)L.comp(r) * p.ld_out + traj] = y[r];
  }
  const long long row = 42LL * p.ld_out;
  bool finite = true;
  WarpCoef<ORDER> cf(threadIdx.x & 31);
  for (int idx = 0; idx < p.n - 1; ++idx) {
    const double h = p.t_vals[idx + 1] - p.t_vals[idx];
    cf.set_step(h);
    double yn[NC];
    rk_fixed_step<ORDER>(L, y, cf, p.mu, p.dir, yn);
#pragma unroll
    for (int r = 0; r < NC; ++r) {
      y[r] = yn[r];
      finite = finite && finite_bits(yn[r]);
    }
    if (writes && (idx + 1) % p.out_every == 0) {
      double* o = p.out + (long long)((idx + 1) / p.out_every) * row;
#pragma unroll
      for (int r = 0; r < NC; ++r) o[(long long)L.comp(r) * p.ld_out + traj] = y[r];
    }
    if (L.broken) break;
  }
  return finite;
}

// Blocks of 2P warps (P = blockDim.x / 64 pairs): warps 0..P-1 are the state
// warps of pairs 0..P-1, warps P..2P-1 their STM warps, so each warp of a
// four-warp block lands on its own sub-partition.
template <int ORDER>
__global__ void __launch_bounds__(128) fixed_rk_pair_kernel(FixedParams p) {
  __shared__ PairLink links[2];
  const int w = threadIdx.x >> 5;
  const int npairs = blockDim.x >> 6;
  const int pair = w % npairs;
  const bool stm = w >= npairs;
  const int lane = threadIdx.x & 31;
  PairLink* lk = &links[pair];
  if (threadIdx.x < npairs * (int)kPairSlots) {
    PairLink* l = &links[threadIdx.x / kPairSlots];
    const int s = threadIdx.x % kPairSlots;
    mbar_init(&l->full[s], 32);
    mbar_init(&l->empty[s], 32);
    if (s == 0) l->broken = 0;
  }
  __syncthreads();
  const PairLane pl(lane);
  const int group = blockIdx.x * npairs + pair;
  const bool active = group * kPairTraj < p.N;  // uniform over the pair's two warps
  const int traj = group * kPairTraj + pl.t;
  const bool valid = active && traj < p.N;
  const int tc = valid ? traj : (active ? p.N - 1 : 0);
  bool finite = true, broken = false;
  if (active) {
    if (!stm) {
      PairState L;
      L.role = pl.role;
      L.base = pl.base;
      L.t = pl.t;
      L.gmask = pl.gmask;
      L.link = lk;
      L.seq = 0;
      L.broken = false;
      finite = pair_fixed_run<ORDER>(L, p, tc, valid && pl.role < 6);
      broken = L.broken;
      finite = __all_sync(pl.gmask, finite);
    } else {
      PairStm L;
      L.col = pl.role < 6 ? pl.role : 5;
      L.t = pl.t;
      L.role = pl.role;
      L.base = pl.base;
      L.gmask = pl.gmask;
      L.link = lk;
      L.seq = 0;
      L.broken = false;
      finite = pair_fixed_run<ORDER>(L, p, tc, valid && pl.role < 6);
      broken = L.broken;
      finite = __all_sync(pl.gmask, finite);
      if (pl.role == 0) lk->fin[pl.t] = finite ? 1 : 0;
      if (broken && lane == 0) lk->broken = 1;
    }
  }
  __syncthreads();
  if (!stm && valid && pl.role == 0 && p.status) {
    const bool all_fin = finite && lk->fin[pl.t] != 0;
    p.status[traj] = (broken || lk->broken) ? HG_SYNC_TIMEOUT : (all_fin ? HG_OK : HG_NONFINITE);
  }
}

// Three-warp fixed-step RK (42-dim, no event): blocks of 96 threads, warp 0
// the state warp of five trajectories, warps 1 and 2 their STM as half
// columns (PairStmHalf), as dop853_trio_kernel lays them out.  The STM
// warp's stage work is halved and a batch of N trajectories issues 3N / 5
// warps instead of 2N / 5: faster while every SM holds at most one group
// (below about 760 trajectories), level or slower beyond, where two groups'
// six warps share an SM's FP64 unit.  The Hessian ring's "empty" barriers
// take both STM warps' arrivals.
template <int ORDER>
__global__ void __launch_bounds__(96) fixed_rk_trio_kernel(FixedParams p) {
  __shared__ PairLink link;
  __shared__ int fin_half[kPairTraj][2];
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < (int)kPairSlots) {
    mbar_init(&link.full[threadIdx.x], 32);
    mbar_init(&link.empty[threadIdx.x], 64);
    if (threadIdx.x == 0) link.broken = 0;
  }
  if (threadIdx.x < 2 * kPairTraj) fin_half[threadIdx.x >> 1][threadIdx.x & 1] = 1;
  __syncthreads();
  const PairLane pl(lane);
  const int group = blockIdx.x;
  const bool active = group * kPairTraj < p.N;  // uniform over the block
  const int hg = 5 * (w - 1) + pl.t;            // STM warps: half-group 0..9
  const int tg = w == 0 ? pl.t : hg / 2;
  const int traj = group * kPairTraj + tg;
  const bool valid = active && traj < p.N;
  const int tc = valid ? traj : (active ? p.N - 1 : 0);
  bool finite = true, broken = false;
  if (active) {
    if (w == 0) {
      PairState L;
      L.role = pl.role;
      L.base = pl.base;
      L.t = pl.t;
      L.gmask = pl.gmask;
      L.link = &link;
      L.seq = 0;
      L.broken = false;
      finite = pair_fixed_run<ORDER>(L, p, tc, valid && pl.role < 6);
      broken = L.broken;
      finite = __all_sync(pl.gmask, finite);
    } else {
      PairStmHalf L;
      L.t = tg;
      L.half = hg & 1;
      L.role = pl.role;
      L.base = pl.base;
      L.gmask = pl.gmask;
      L.link = &link;
      L.seq = 0;
      L.broken = false;
      finite = pair_fixed_run<ORDER>(L, p, tc, valid && pl.role < 6);
      broken = L.broken;
      finite = __all_sync(pl.gmask, finite);
      if (pl.role == 0) fin_half[tg][hg & 1] = finite ? 1 : 0;
      if (broken && lane == 0) link.broken = 1;
    }
  }
  __syncthreads();
  if (w == 0 && valid && pl.role == 0 && p.status) {
    const bool all_fin = finite && fin_half[pl.t][0] != 0 && fin_half[pl.t][1] != 0;
    p.status[traj] = (broken || link.broken) ? HG_SYNC_TIMEOUT : (all_fin ? HG_OK : HG_NONFINITE);
  }
}

// ---------------------------------------------------------------------------
// DOP853 on the paired warps (42-dim, single pass, no event; rk.py:2375-2549)
// ---------------------------------------------------------------------------
// Besides the Hessian hand-off, the step-size control needs norms over all
// 42 components: both warps store their components of two vectors (and one
// flag each) in a per-trajectory gather slot, meet at a two-warp barrier (an
// mbarrier with 64 arrivals, two slots alternating by exchange), and every
// lane then forms the same numpy-order dots -- so both warps take the same
// accept / reject decisions, step sizes and dense-output samples.  Each warp
// loops while any of its five trajectories is running; finished ones keep
// computing on their frozen state without committing anything, so every
// hand-off has all 32 lanes of both warps.
struct PairGather {
  // slot, trajectory, vector, 42 components + flags: [42] the state warp's,
  // [43], [44] the STM's (one warp: both; two half-column warps: one each)
  double v[2][kPairTraj][2][45];
  unsigned long long bar[2];
};

template <class LT>
__device__ __forceinline__ void pair_exchange(const LT& L, PairGather* gx, unsigned& gseq,
                                              const double (&a)[LT::NC], const double (&b)[LT::NC],
                                              double flag, double& dot_a, double& dot_b, double& flag_all) {
  const unsigned sl = gseq & 1u;
  double* va = gx->v[sl][L.t][0];
  double* vb = gx->v[sl][L.t][1];
  if (!L.broken) {
    if (L.role < 6) {
#pragma unroll
      for (int r = 0; r < LT::NC; ++r) {
        va[L.comp(r)] = a[r];
        vb[L.comp(r)] = b[r];
      }
      if (L.role == 0) {
        va[L.flag_slot()] = flag;
        if constexpr (LT::kState == false && LT::NC == 6) va[44] = flag;
      }
    }
    mbar_arrive(&gx->bar[sl]);
    const bool ok = mbar_wait(&gx->bar[sl], (gseq >> 1) & 1u);
    L.broken = !__all_sync(0xFFFFFFFFu, ok);
  }
  ++gseq;
  dots42_group(L, va, vb, dot_a, dot_b);
  flag_all = (va[42] != 0.0 && va[43] != 0.0 && va[44] != 0.0) ? 1.0 : 0.0;
}

// One warp's part of the DOP853 propagation of its five trajectories.
// Decisions that set how many hand-offs a step makes (keep stepping, build a
// dense cache) are votes over the warp (BLOCK = false: both warps of a pair
// hold the same trajectories) or over the block (BLOCK = true: the three
// warps of a trio hold different subsets).  Returns its broken flag.
template <bool BLOCK, class LT>
__device__ __forceinline__ bool pair_dop_run(const LT& L, const DopParams& p, PairGather* gx, const double* coef_tab,
                                             int traj, bool valid, bool writes) {
  auto vote_any = [](bool v) -> bool {
    if constexpr (BLOCK)
      return __syncthreads_or(v ? 1 : 0) != 0;
    else
      return __any_sync(0xFFFFFFFFu, v);
  };
  constexpr int NC = LT::NC;
  constexpr int D = 42;
  const double t0 = p.t0_arr ? p.t0_arr[traj] : p.t0;
  const double tmax = p.tmax_arr ? p.tmax_arr[traj] : p.tmax;
  double y[NC];
#pragma unroll
  for (int r = 0; r < NC; ++r) y[r] = p.y0[(long long)L.comp(r) * p.ld + traj];
  double k[13][NC];
  L.rhs(y, p.mu, p.dir, k[0]);
  unsigned gseq = 0;
  double h;
  {
    double a[NC], b[NC];
#pragma unroll
    for (int d = 0; d < NC; ++d) {
      const double scale0 = p.atol + p.rtol * fabs(y[d]);
      a[d] = y[d] / scale0;
      b[d] = k[0][d] / scale0;
    }
    double da, db, unused;
    pair_exchange(L, gx, gseq, a, b, 0.0, da, db, unused);
    const double sn = sqrt((double)D);
    h = select_initial_step(sqrt(da) / sn, sqrt(db) / sn, p.min_step, p.max_step);
  }
  double t = t0, err_prev = -1.0, prev_pow = 0.0;
  int acc = 0, rej = 0;
  const bool dense = p.m >= 2;
  int q_next = (dense && p.dense_last) ? p.m - 1 : 0;
  int status = HG_OK;
  bool running = valid;
  double step_ls = 0.0;
  if (dense) step_ls = (tmax - t0) / (double)(p.m - 1);
  auto sample_t = [&](int q) -> double { return q == p.m - 1 ? tmax : (double)q * step_ls + t0; };
  // integrators/rk.py loop test (t - t_end) * direction < 0, direction +1
  bool live = running && hg_lt0(t - tmax);
  DopGroupCoef<6> cf(coef_tab, L.role % 6, L.base, L.gmask);
  while (vote_any(live)) {
    bool go = live;
    if (go && (long long)(acc + rej) >= p.max_steps) {
      status = HG_MAX_STEPS;
      running = false;
      go = false;
    }
    double hh = h;
    if (go) {
      hh = clamp_step(hh, p.max_step, p.min_step);
      hh = adjust_step_to_endpoint(t, hh, tmax);
    }
    double yh[NC], e5[NC], e3[NC];
    cf.set_step(hh);
    DopLaneT<LT>::step(L, y, cf, hh, p.mu, p.dir, k, yh, e5, e3);
    double s5[NC], s3[NC];
    bool fin = true;
#pragma unroll
    for (int d = 0; d < NC; ++d) {
      const double scale = p.atol + p.rtol * np_maximum_abs(y[d], yh[d]);
      const double is = hg_rcp_rn(scale);
      s5[d] = hg_div_rn(e5[d], scale, is);
      s3[d] = hg_div_rn(e3[d], scale, is);
      fin = fin && finite_bits(yh[d]);
    }
    fin = __all_sync(L.gmask, fin);
    double n5, n3, fin_all;
    pair_exchange(L, gx, gseq, s5, s3, fin ? 1.0 : 0.0, n5, n3, fin_all);
    fin = fin_all != 0.0;
    double err_norm;
    if (hg_both0(n5, n3))
      err_norm = 0.0;
    else
      err_norm = (fabs(hh) * n5) / sqrt((n5 + 0.01 * n3) * (double)D);
    const bool accepted = hg_le_pos(err_norm, HG_BITS_1);  // err_norm <= 1
    const double t_new = t + hh;
    // dense samples inside (t, t_new] (reference: searchsorted on nodes);
    // the cache's three extra evaluations run on the whole warp
    bool need = false, last = false;
    if (go && accepted && dense) {
      last = !(t_new - tmax < 0.0);
      need = q_next < p.m && (last || sample_t(q_next) < t_new);
    }
    if (vote_any(need)) {
      const double hseg = t_new - t;
      double F[7][NC];
      DopLaneT<LT>::dense_cache(L, y, yh, hseg, p.mu, p.dir, k, F);
      if (need) {
        while (q_next < p.m && (last || sample_t(q_next) < t_new)) {
          const double x = (sample_t(q_next) - t) / hseg;
          if (writes) {
            double* o = p.y_out + (long long)(p.dense_last ? 0 : q_next) * D * p.ld;
#pragma unroll
            for (int d = 0; d < NC; ++d) o[(long long)L.comp(d) * p.ld + traj] = DopLaneT<LT>::eval1(y[d], F, d, x);
          }
          ++q_next;
        }
      }
    }
    if (go) {
      if (accepted) {
        ++acc;
        t = t_new;
#pragma unroll
        for (int d = 0; d < NC; ++d) {
          y[d] = yh[d];
          k[0][d] = k[12][d];
        }
      } else {
        ++rej;
      }
      h = hh * pi_factor(L, accepted, err_norm, err_prev, prev_pow);
      if (accepted) {
        err_prev = err_norm;
        if (!fin) {
          status = HG_NONFINITE;
          running = false;
        }
      } else {
        h = clamp_step(h, p.max_step, p.min_step);
      }
    }
    live = running && hg_lt0(t - tmax) && !L.broken;
  }
  if (valid && writes) {
    // the reference's dense output falls back to the single stored node when
    // no step was taken
    if (dense) {
      while (q_next < p.m) {
        double* o = p.y_out + (long long)(p.dense_last ? 0 : q_next) * D * p.ld;
#pragma unroll
        for (int d = 0; d < NC; ++d) o[(long long)L.comp(d) * p.ld + traj] = y[d];
        ++q_next;
      }
    }
    if (p.y_end) {
#pragma unroll
      for (int d = 0; d < NC; ++d) p.y_end[(long long)L.comp(d) * p.ld + traj] = y[d];
    }
    if (LT::kState && L.role == 0) {
      if (p.t_end) p.t_end[traj] = t;
      if (p.n_accept) p.n_accept[traj] = acc;
      if (p.n_reject) p.n_reject[traj] = rej;
      if (p.status) p.status[traj] = status;
    }
  }
  return L.broken;
}

// Blocks of one or two pairs, laid out as fixed_rk_pair_kernel's.
static __global__ void __launch_bounds__(128) dop853_pair_kernel(DopParams p) {
  __shared__ PairLink links[2];
  __shared__ PairGather gathers[2];
  __shared__ double coef_tab[dop_nnz()];
  dop_coef_table_init(coef_tab);
  const int w = threadIdx.x >> 5;
  const int npairs = blockDim.x >> 6;
  const int pair = w % npairs;
  const bool stm = w >= npairs;
  const int lane = threadIdx.x & 31;
  PairLink* lk = &links[pair];
  PairGather* gx = &gathers[pair];
  if (threadIdx.x < npairs * (int)kPairSlots) {
    PairLink* l = &links[threadIdx.x / kPairSlots];
    const int s = threadIdx.x % kPairSlots;
    mbar_init(&l->full[s], 32);
    mbar_init(&l->empty[s], 32);
    if (s == 0) l->broken = 0;
    if (s < 2) mbar_init(&gathers[threadIdx.x / kPairSlots].bar[s], 64);
  }
  __syncthreads();
  const PairLane pl(lane);
  const int group = blockIdx.x * npairs + pair;
  // list mode (n_in given): the trajectories 0 .. *n_in - 1 of a launch sized
  // for p.N run; the others' blocks return at once
  const int N = p.n_in ? *p.n_in : p.N;
  const bool active = group * kPairTraj < N;  // uniform over the pair's two warps
  const int traj = group * kPairTraj + pl.t;
  const bool valid = active && traj < N;
  const int tc = valid ? traj : (active ? N - 1 : 0);
  bool broken = false;
  if (active) {
    if (!stm) {
      PairState L;
      L.role = pl.role;
      L.base = pl.base;
      L.t = pl.t;
      L.gmask = pl.gmask;
      L.link = lk;
      L.seq = 0;
      L.broken = false;
      broken = pair_dop_run<false>(L, p, gx, coef_tab, tc, valid, valid && pl.role < 6);
    } else {
      PairStm L;
      L.col = pl.role < 6 ? pl.role : 5;
      L.t = pl.t;
      L.role = pl.role;
      L.base = pl.base;
      L.gmask = pl.gmask;
      L.link = lk;
      L.seq = 0;
      L.broken = false;
      broken = pair_dop_run<false>(L, p, gx, coef_tab, tc, valid, valid && pl.role < 6);
      if (broken && lane == 0) lk->broken = 1;
    }
  }
  __syncthreads();
  if (!stm && valid && pl.role == 0 && p.status && (broken || lk->broken)) p.status[traj] = HG_SYNC_TIMEOUT;
}

// Three-warp DOP853 (42-dim, single pass, no event): blocks of 96 threads,
// warp 0 the state warp of five trajectories, warps 1 and 2 their STM as
// half-columns (PairStmHalf) -- the STM warp's stage work halved, for
// batches too small to fill the GPU, where one warp's step sets the time.
// The Hessian ring's "empty" barriers take both STM warps' arrivals, the
// norm gather all three warps'.
static __global__ void __launch_bounds__(96) dop853_trio_kernel(DopParams p) {
  __shared__ PairLink link;
  __shared__ PairGather gather;
  __shared__ double coef_tab[dop_nnz()];
  dop_coef_table_init(coef_tab);
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < (int)kPairSlots) {
    mbar_init(&link.full[threadIdx.x], 32);
    mbar_init(&link.empty[threadIdx.x], 64);
    if (threadIdx.x < 2) mbar_init(&gather.bar[threadIdx.x], 96);
    if (threadIdx.x == 0) link.broken = 0;
  }
  __syncthreads();
  const PairLane pl(lane);
  const int group = blockIdx.x;
  // list mode (n_in given): the trajectories 0 .. *n_in - 1 run
  const int N = p.n_in ? *p.n_in : p.N;
  const bool active = group * kPairTraj < N;  // uniform over the block
  // trajectory of this lane within the group
  const int hg = 5 * (w - 1) + pl.t;                 // STM warps: half-group 0..9
  const int tg = w == 0 ? pl.t : hg / 2;
  const int traj = group * kPairTraj + tg;
  const bool valid = active && traj < N;
  const int tc = valid ? traj : (active ? N - 1 : 0);
  bool broken = false;
  if (active) {
    if (w == 0) {
      PairState L;
      L.role = pl.role;
      L.base = pl.base;
      L.t = pl.t;
      L.gmask = pl.gmask;
      L.link = &link;
      L.seq = 0;
      L.broken = false;
      broken = pair_dop_run<true>(L, p, &gather, coef_tab, tc, valid, valid && pl.role < 6);
    } else {
      PairStmHalf L;
      L.t = tg;
      L.half = hg & 1;
      L.role = pl.role;
      L.base = pl.base;
      L.gmask = pl.gmask;
      L.link = &link;
      L.seq = 0;
      L.broken = false;
      broken = pair_dop_run<true>(L, p, &gather, coef_tab, tc, valid, valid && pl.role < 6);
      if (broken && lane == 0) link.broken = 1;
    }
  }
  __syncthreads();
  if (w == 0 && valid && pl.role == 0 && p.status && (broken || link.broken)) p.status[traj] = HG_SYNC_TIMEOUT;
}

}  // namespace hg
