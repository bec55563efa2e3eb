// C ABI of the propagation library (declarations and contracts in
// include/hitengpu.h).  Owns the per-handle scratch: the lane-refill
// counters and the pinned live-count word (allocated in hg_create), the
// record pool of deferred event refinement and the corrector's buffers
// (sized by hg_reserve / hg_reserve_correct, or grown on first use); every
// allocation is counted (HG_COUNTER_ALLOCATIONS).
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "hg_internal.h"
#include "hg_kernels.cuh"
#include "hg_pair.cuh"
#include "hitengpu.h"

struct hg_handle {
  int device = 0;
  int sm_count = 0;
  int* counters = nullptr;  // scratch: lane-refill counters
  int block = 32;           // threads per block (32, 64 or 128)
  int lanes_d6 = 0;         // lanes per 6-dim DOP853 trajectory: 0 auto, 1, 2, 6
  int lanes_d42 = 0;        // lanes per 42-dim trajectory: 0 auto, 7, 14, 12 (paired warps, fixed RK)
  int sm_capacity_x10 = 30;  // warps' FP64 demand an SM serves at full speed, x10 (layout cost models)
  long long refine_pool_max = 8LL << 30;  // largest record pool a single-pass call allocates (bytes)
  int seg_steps = 16;       // attempted steps per segment of the scheduled DOP853 driver
  int spread = 0;           // 1: DOP853 blocks of 4 warps, one block per SM (one warp per sub-partition)
  int smem_per_sm = 0;      // bytes of shared memory per SM
  int* host_count = nullptr;  // pinned: live-trajectory count read back between segments
  char* scratch = nullptr;    // grow-only: saved crossing steps of single-pass calls
  long long scratch_bytes = 0;
  char* corr = nullptr;       // grow-only: device buffers of hg_correct_halo
  long long corr_bytes = 0;
  void* corr_graph = nullptr;            // the device corrector's instantiated graph and its key
  void (*corr_graph_free)(void*) = nullptr;
  long long launches = 0;   // kernels launched through this handle
  long long allocs = 0;     // device and pinned-host allocations made for this handle
  char err[512] = {0};
};

namespace {

int fail(hg_handle* h, int code, const char* fmt, ...) {
  if (h) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(h->err, sizeof(h->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

int check_launch(hg_handle* h, const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(h, HG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  ++h->launches;
  return HG_OK;
}

hg::Dir make_dir(int dim, int fwd, int flip_lo, int flip_hi) {
  hg::Dir d;
  if (fwd == -1) {
    d.neg_lo = flip_lo;
    d.neg_hi = flip_hi;
  } else {
    d.neg_lo = 0;
    d.neg_hi = 0;
  }
  (void)dim;
  return d;
}

// Blocks default to one warp: small batches then spread over all SMs.

template <int ORDER, int G>
int launch_fixed(hg_handle* h, const hg::FixedParams& p, cudaStream_t s) {
  const int tpb = (h->block / 32) * hg::Layout<G>::TPW;  // trajectories per block
  const int grid = (p.N + tpb - 1) / tpb;
  if (grid > 0) {
    if constexpr (G == 14) {
      hg::fixed_rk_kernel<ORDER, G><<<grid, h->block, 0, s>>>(p);
    } else {
      if (p.ev_index >= 0)
        hg::fixed_rk_event_kernel<ORDER, G><<<grid, h->block, 0, s>>>(p);
      else
        hg::fixed_rk_kernel<ORDER, G><<<grid, h->block, 0, s>>>(p);
    }
  }
  return check_launch(h, "fixed_rk_kernel");
}

// Lanes per 42-dim trajectory: 7 (an STM column per lane) or 14 (half a
// column per lane: half the stage work per lane, twice the warps).  Unless
// fixed by tuning, the one with the least time per step, where a warp's step
// takes lat(G) (G = 14: 0.65 of G = 7) while its SM holds at most three
// warps' FP64 demand, beyond which warps share the SM's FP64 unit.  With
// `pair` the paired-warp layout (12 lanes on two warps, five trajectories
// per pair, lat 0.6: RK8 on GB300, 125 ms against 214 ms for G = 7 over 3000
// steps of 512 states) competes too.
int lanes_d42(const hg_handle* h, int n, bool pair = false, double pair_lat = 0.0) {
  if (h->lanes_d42 != 0) return ((h->lanes_d42 == 12 || h->lanes_d42 == 18) && !pair) ? 7 : h->lanes_d42;
  const double cap = 0.1 * h->sm_capacity_x10 * h->sm_count;
  const double w7 = (double)((n + 3) / 4), w14 = (double)((n + 1) / 2);
  const double wp = 2.0 * (double)((n + hg::kPairTraj - 1) / hg::kPairTraj);
  const double c7 = 1.0 * (w7 > cap ? w7 / cap : 1.0);
  const double c14 = 0.65 * (w14 > cap ? w14 / cap : 1.0);
  const double cp = pair_lat * (wp > cap ? wp / cap : 1.0);
  if (pair && pair_lat > 0.0 && cp < c7 && cp < c14) return 12;
  return c14 < c7 ? 14 : 7;
}

// Per-step latency of the paired-warp layout relative to G = 7 (0: not
// chosen automatically).
constexpr double kPairLatFixed = 0.6;
// Event-free single-pass DOP853 on 42 components: the three-warp layout
// (state warp + two half-column STM warps) while its warps fit about three
// per SM (3 N / 5 <= 3 x SMs), the pair above -- measured for the corrector's
// STM legs (ms: 64 orbits trio 1.60, pair 1.81, G = 14 1.91, G = 7 2.43; 512
// orbits 1.68 / 1.88 / 1.95 / 2.53; 2048 orbits 2.91 / 2.66 / 3.42 / 2.97)
// and one trajectory with 2000 dense samples (7.4 / 10.6 / 9.3 / 15.0).
int lanes_d42_dop_free(const hg_handle* h, int n) {
  if (h->lanes_d42 != 0) return h->lanes_d42;
  const double cap = 0.1 * h->sm_capacity_x10 * h->sm_count;
  return 3.0 * ((n + hg::kPairTraj - 1) / hg::kPairTraj) <= cap ? 18 : 12;
}

// Paired-warp DOP853 launch (42-dim, no event, single pass): blocks of one
// pair (two with HG_TUNE_BLOCK_THREADS 128).
int launch_dop853_trio(hg_handle* h, const hg::DopParams& p, cudaStream_t s) {
  const int grid = (p.N + hg::kPairTraj - 1) / hg::kPairTraj;
  if (grid < 1) return HG_OK;
  hg::dop853_trio_kernel<<<grid, 96, 0, s>>>(p);
  return check_launch(h, "dop853_trio_kernel");
}

int launch_dop853_pair(hg_handle* h, const hg::DopParams& p, cudaStream_t s) {
  const int block = h->block >= 128 ? 128 : 64;
  const int per_block = (block / 64) * hg::kPairTraj;
  const int grid = (p.N + per_block - 1) / per_block;
  if (grid < 1) return HG_OK;
  hg::dop853_pair_kernel<<<grid, block, 0, s>>>(p);
  return check_launch(h, "dop853_pair_kernel");
}

// Paired-warp fixed-step launch: blocks of two pairs (four warps, one per
// sub-partition; HG_TUNE_BLOCK_THREADS 128) or of one pair (64: the pairs
// spread over more SMs); while four-warp blocks fit one per SM, each reserves
// more than half of the SM's shared memory so that no two share an SM.
template <int ORDER>
int launch_fixed_pair(hg_handle* h, const hg::FixedParams& p, cudaStream_t s) {
  const int block = h->block >= 128 ? 128 : 64;
  const int per_block = (block / 64) * hg::kPairTraj;
  const int grid = (p.N + per_block - 1) / per_block;
  if (grid < 1) return HG_OK;
  size_t smem = 0;
  if (block == 128 && grid <= h->sm_count && h->smem_per_sm > 0) {
    smem = (size_t)(h->smem_per_sm / 2 + 1024);
    if (cudaFuncSetAttribute(hg::fixed_rk_pair_kernel<ORDER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess) {
      cudaGetLastError();
      smem = 0;
    }
  }
  hg::fixed_rk_pair_kernel<ORDER><<<grid, block, smem, s>>>(p);
  return check_launch(h, "fixed_rk_pair_kernel");
}

// Three-warp fixed-step launch: one block of 96 threads per five trajectories.
template <int ORDER>
int launch_fixed_trio(hg_handle* h, const hg::FixedParams& p, cudaStream_t s) {
  const int grid = (p.N + hg::kPairTraj - 1) / hg::kPairTraj;
  if (grid < 1) return HG_OK;
  hg::fixed_rk_trio_kernel<ORDER><<<grid, 96, 0, s>>>(p);
  return check_launch(h, "fixed_rk_trio_kernel");
}

int fixed_common(hg_handle* h, double mu, int order, int dim, int N, const double* y0, long long ld_in,
                 const double* t_vals, int n_nodes, int out_every, double* y_out, long long ld_out, int fwd,
                 int flip_lo, int flip_hi, int* status, hg::FixedParams& p) {
  if (order != 4 && order != 6 && order != 8) return fail(h, HG_ERR_ARGS, "order must be 4, 6 or 8 (got %d)", order);
  if (dim != 6 && dim != 42) return fail(h, HG_ERR_ARGS, "dim must be 6 or 42 (got %d)", dim);
  if (N < 0 || n_nodes < 1 || out_every < 1) return fail(h, HG_ERR_ARGS, "bad sizes");
  if (ld_in < N || ld_out < N) return fail(h, HG_ERR_ARGS, "leading dimension < N");
  if (N > 0 && (!y0 || !t_vals || !y_out)) return fail(h, HG_ERR_ARGS, "null array");
  if (flip_lo < 0 || flip_hi > dim || flip_lo > flip_hi) return fail(h, HG_ERR_ARGS, "bad flip range");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, HG_ERR_CUDA, "cudaSetDevice");
  memset(&p, 0, sizeof(p));
  p.N = N;
  p.mu = mu;
  p.dir = make_dir(dim, fwd, flip_lo, flip_hi);
  p.y0 = y0;
  p.ld_in = ld_in;
  p.t_vals = t_vals;
  p.n = n_nodes;
  p.out_every = out_every;
  p.out = y_out;
  p.ld_out = ld_out;
  p.status = status;
  p.ev_index = -1;
  return HG_OK;
}

int fixed_dispatch(hg_handle* h, int order, int dim, const hg::FixedParams& p, cudaStream_t s) {
  if (dim == 6) {
    if (order == 4) return launch_fixed<4, 1>(h, p, s);
    if (order == 6) return launch_fixed<6, 1>(h, p, s);
    return launch_fixed<8, 1>(h, p, s);
  }
  const int g42 = p.ev_index < 0 ? lanes_d42(h, p.N, true, kPairLatFixed) : 7;
  if (g42 == 18) {
    if (order == 4) return launch_fixed_trio<4>(h, p, s);
    if (order == 6) return launch_fixed_trio<6>(h, p, s);
    return launch_fixed_trio<8>(h, p, s);
  }
  if (g42 == 12) {
    if (order == 4) return launch_fixed_pair<4>(h, p, s);
    if (order == 6) return launch_fixed_pair<6>(h, p, s);
    return launch_fixed_pair<8>(h, p, s);
  }
  if (g42 == 14) {
    if (order == 4) return launch_fixed<4, 14>(h, p, s);
    if (order == 6) return launch_fixed<6, 14>(h, p, s);
    return launch_fixed<8, 14>(h, p, s);
  }
  if (order == 4) return launch_fixed<4, 7>(h, p, s);
  if (order == 6) return launch_fixed<6, 7>(h, p, s);
  return launch_fixed<8, 7>(h, p, s);
}

// Record pool of the deferred event refinement for N trajectories of
// dimension D with up to max_hits crossings each: count (256 B), trajectory
// and hit index per record, records ((15 D + 3) doubles each), all for
// N * max_hits records.
long long refine_area_bytes(int N, int D, int max_hits) {
  auto up = [](long long x) { return (x + 255) & ~255LL; };
  if (max_hits < 1) return 0;
  const long long cap = (long long)N * max_hits;
  return 256 + 2 * up(cap * 4) + up((15LL * D + 3) * cap * 8);
}

void refine_area_carve(int N, int max_hits, char* base, hg::DopParams& p) {
  auto up = [](long long x) { return (x + 255) & ~255LL; };
  const long long cap = (long long)N * max_hits;
  p.refine_count = (int*)base;
  p.refine_list = (int*)(base + 256);
  p.refine_hit = (int*)(base + 256 + up(cap * 4));
  p.rec = (double*)(base + 256 + 2 * up(cap * 4));
  p.rec_ld = cap;
}

// Event crossings are refined after the integration, in lock step.
bool defer_refine(const hg::DopParams& p) { return p.ev_index >= 0 && p.max_hits >= 1; }

template <int G>
int launch_refine(hg_handle* h, hg::DopParams p, cudaStream_t s) {
  const int kBlock = h->block;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hg::refine_kernel<G>, kBlock, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int tpb = (kBlock / 32) * hg::Layout<G>::TPW;
  const long long records = p.rec_ld;
  const long long need = (records + tpb - 1) / tpb;
  const int cap = per_sm * h->sm_count;
  const int grid = need < cap ? (int)need : cap;
  if (grid < 1) return HG_OK;
  p.stride = grid * tpb;
  hg::refine_kernel<G><<<grid, kBlock, 0, s>>>(p);
  return check_launch(h, "refine_kernel");
}

int refine_pending(hg_handle* h, const hg::DopParams& p, int dim, cudaStream_t s) {
  if (!p.rec) return HG_OK;
  return dim == 6 ? launch_refine<1>(h, p, s) : launch_refine<7>(h, p, s);
}

// Grow-only device buffer of the handle: a no-op (no allocation) when it
// already holds `bytes`.  `slack` adds a quarter for buffers sized per call.
int grow(hg_handle* h, char** buf, long long* have, long long bytes, bool slack, const char* what) {
  if (bytes <= *have) return HG_OK;
  if (*buf) cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  const long long want = slack ? bytes + bytes / 4 : bytes;
  if (cudaMalloc(buf, (size_t)want) != cudaSuccess) {
    *buf = nullptr;
    return fail(h, HG_ERR_CUDA, "cudaMalloc of %lld bytes of %s failed", want, what);
  }
  ++h->allocs;
  *have = want;
  return HG_OK;
}

int ensure_scratch(hg_handle* h, long long bytes) {
  return grow(h, &h->scratch, &h->scratch_bytes, bytes, true, "refinement scratch");
}

// Launch shape of a DOP853 kernel: threads per block, dynamic shared memory
// and resident blocks per SM.  In spread mode a block of four warps reserves
// more than half of the SM's shared memory (unused), so no two blocks share
// an SM: four warps per SM, which share its FP64 unit at nearly the rate of
// one warp each.
struct Shape {
  int block;
  size_t smem;
  int per_sm;
};

template <class K>
Shape dop_shape(const hg_handle* h, K kernel) {
  Shape sh{h->block, 0, 1};
  if (h->spread && h->smem_per_sm > 0) {
    sh.block = 128;
    sh.smem = (size_t)(h->smem_per_sm / 2 + 1024);
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem) != cudaSuccess) {
      cudaGetLastError();
      sh.block = h->block;
      sh.smem = 0;
    }
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, sh.block, sh.smem) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  sh.per_sm = per_sm;
  return sh;
}

template <int G>
int launch_dop853(hg_handle* h, hg::DopParams p, cudaStream_t s) {
  if (p.N <= 0) return HG_OK;
  // launches without dense samples run the kernel built without that path
  auto kern = p.m >= 2 ? hg::dop853_kernel<G, true> : hg::dop853_kernel<G, false>;
  const Shape sh = dop_shape(h, kern);
  const int kBlock = sh.block;
  const int per_sm = sh.per_sm;
  cudaError_t e;
  const int tpb = (kBlock / 32) * hg::Layout<G>::TPW;
  const int need = (p.N + tpb - 1) / tpb;
  const int cap = per_sm * h->sm_count;
  const int grid = need < cap ? need : cap;
  p.stride = grid * tpb;
  p.next_traj = nullptr;
  if (need > cap) {
    p.next_traj = h->counters;
    e = cudaMemsetAsync(h->counters, 0, sizeof(int), s);
    if (e != cudaSuccess) return fail(h, HG_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
  }
  kern<<<grid, kBlock, sh.smem, s>>>(p);
  return check_launch(h, "dop853_kernel");
}

// Lanes per 6-dim DOP853 trajectory when the caller did not choose: the
// largest group whose warps still fit four per SM, about what an SM's FP64
// unit serves at each warp's full rate (the longest trajectory sets the time
// and its per-step latency falls with the group size), single lanes once even
// those oversubscribe.
int auto_lanes_d6(const hg_handle* h, int N) {
  const long long smsp = 4LL * h->sm_count;
  if ((N + 4LL) / 5 <= smsp) return 6;
  if ((N + 15LL) / 16 <= smsp) return 2;
  return 1;
}

__global__ void seg_init_kernel(int N, int* list, int* count, int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    list[i] = i;
    status[i] = -2;  // not started
  }
  if (i == 0) *count = N;
}

// Workspace of the segmented DOP853 driver, carved from one caller buffer.
struct SegWs {
  int* list[2];
  int* count;  // [2]
  double* h;
  double* err_prev;
  double* prev_pow;
  int* q;
  char* refine;  // saved crossing steps (refine_area_bytes)
};

long long seg_ws_layout(int N, int D, int max_hits, char* base, SegWs* w) {
  auto up = [](long long x) { return (x + 255) & ~255LL; };
  long long off = 0;
  const long long ni = up((long long)N * 4), nd = up((long long)N * 8);
  if (w) w->list[0] = (int*)(base + off);
  off += ni;
  if (w) w->list[1] = (int*)(base + off);
  off += ni;
  if (w) w->count = (int*)(base + off);
  off += 256;
  if (w) w->h = (double*)(base + off);
  off += nd;
  if (w) w->err_prev = (double*)(base + off);
  off += nd;
  if (w) w->prev_pow = (double*)(base + off);
  off += nd;
  if (w) w->q = (int*)(base + off);
  off += ni;
  if (w) w->refine = base + off;
  off += refine_area_bytes(N, D, max_hits);
  return off;
}

// One segment over the live list list[a] (at most n_live entries): every
// live trajectory advances by up to seg_steps attempted steps; those still
// running are appended to list[a ^ 1].
template <int G>
int launch_segment(hg_handle* h, hg::DopParams p, const SegWs& w, int seg_steps, int a, int n_live, cudaStream_t s) {
  auto kern = p.m >= 2 ? hg::dop853_kernel<G, true> : hg::dop853_kernel<G, false>;
  const Shape sh = dop_shape(h, kern);
  const int kBlock = sh.block;
  const int per_sm = sh.per_sm;
  const int tpb = (kBlock / 32) * hg::Layout<G>::TPW;
  const int need = (n_live + tpb - 1) / tpb;
  const int cap = per_sm * h->sm_count;
  const int grid = need < cap ? need : cap;
  const int b = a ^ 1;
  if (cudaMemsetAsync(w.count + b, 0, sizeof(int), s) != cudaSuccess) return fail(h, HG_ERR_CUDA, "memset");
  if (grid < 1) return HG_OK;
  p.stride = grid * tpb;
  p.next_traj = nullptr;
  p.seg = 1;
  p.seg_steps = seg_steps;
  p.ws_h = w.h;
  p.ws_err_prev = w.err_prev;
  p.ws_prev_pow = w.prev_pow;
  p.ws_q = w.q;
  p.active_in = w.list[a];
  p.n_in = w.count + a;
  p.active_out = w.list[b];
  p.n_out = w.count + b;
  kern<<<grid, kBlock, sh.smem, s>>>(p);
  return check_launch(h, "dop853_kernel (segment)");
}

int seg_init(hg_handle* h, const hg::DopParams& p, const SegWs& w, cudaStream_t s) {
  seg_init_kernel<<<(p.N + 255) / 256, 256, 0, s>>>(p.N, w.list[0], w.count, p.status);
  return check_launch(h, "seg_init_kernel");
}

template <int G>
int launch_dop853_seg(hg_handle* h, hg::DopParams p, const SegWs& w, int seg_steps, int max_segments, int resume,
                      cudaStream_t s) {
  if (!resume) {
    const int rc = seg_init(h, p, w, s);
    if (rc != HG_OK) return rc;
  }
  for (int sgm = 0; sgm < max_segments; ++sgm) {
    const int rc = launch_segment<G>(h, p, w, seg_steps, sgm & 1, p.N, s);
    if (rc != HG_OK) return rc;
  }
  if (max_segments & 1) {  // leave the live list in list[0] for a resume
    if (cudaMemcpyAsync(w.list[0], w.list[1], sizeof(int) * (size_t)p.N, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(w.count, w.count + 1, sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return fail(h, HG_ERR_CUDA, "memcpy");
  }
  return HG_OK;
}

// Layout of the next segment of a 6-dim batch with n_live trajectories
// left: the group size with the least time per step.  One warp's step takes
// lat(G) while its SM is not saturated (measured on GB300 for the longest
// manifold trajectory: 75.4, 46.9 and 30.2 us for G = 1, 2, 6); an SM's FP64
// unit serves about three such warps at full speed (two run as fast as one,
// four lose ~13 %), beyond which they share it.
int sched_lanes_d6(const hg_handle* h, int n_live) {
  if (h->lanes_d6 != 0) return h->lanes_d6;
  const double smsp = 0.1 * h->sm_capacity_x10 * h->sm_count;
  const int gs[3] = {1, 2, 6};
  const int tpw[3] = {32, 16, 5};
  const double lat[3] = {1.0, 0.622, 0.400};
  int best = 0;
  double best_cost = 0.0;
  for (int i = 0; i < 3; ++i) {
    const double warps = (double)((n_live + tpw[i] - 1) / tpw[i]);
    const double load = warps / smsp;
    const double cost = lat[i] * (load > 1.0 ? load : 1.0);
    if (i == 0 || cost < best_cost) {
      best = i;
      best_cost = cost;
    }
  }
  return gs[best];
}

__global__ void fp64_probe_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-9, x2 = x0 + 2e-9, x3 = x0 + 3e-9;
  double x4 = x0 + 4e-9, x5 = x0 + 5e-9, x6 = x0 + 6e-9, x7 = x0 + 7e-9;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 1.2345) out[0] = s;  // keeps the chains alive
}

}  // namespace

extern "C" {

const char* hg_version(void) { return "hitengpu 0.1 (sm_103a, FP64)"; }

int hg_create(const hg_config* cfg, hg_handle** out) {
  if (!out) return HG_ERR_ARGS;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return HG_ERR_NO_DEVICE;
  hg_handle* h = new (std::nothrow) hg_handle();
  if (!h) return HG_ERR_ARGS;
  h->device = cfg ? cfg->device : 0;
  if (h->device < 0 || h->device >= ndev) {
    delete h;
    return HG_ERR_ARGS;
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device);
  cudaDeviceGetAttribute(&h->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, h->device);
  cudaError_t e = cudaMalloc(&h->counters, 64 * sizeof(int));
  if (e == cudaSuccess) {
    ++h->allocs;
    e = cudaHostAlloc(&h->host_count, sizeof(int), cudaHostAllocDefault);
    if (e == cudaSuccess) ++h->allocs;
    else h->host_count = nullptr;
  }
  cudaSetDevice(prev);
  if (e != cudaSuccess) {
    if (h->counters) cudaFree(h->counters);
    delete h;
    return HG_ERR_CUDA;
  }
  *out = h;
  return HG_OK;
}

int hg_destroy(hg_handle* h) {
  if (!h) return HG_OK;
  if (h->counters) cudaFree(h->counters);
  if (h->host_count) cudaFreeHost(h->host_count);
  if (h->scratch) cudaFree(h->scratch);
  if (h->corr) cudaFree(h->corr);
  if (h->corr_graph && h->corr_graph_free) h->corr_graph_free(h->corr_graph);
  delete h;
  return HG_OK;
}

int hg_reserve(hg_handle* h, int max_N, int dim, int max_hits) {
  if (!h) return HG_ERR_ARGS;
  if (max_N < 0 || (dim != 6 && dim != 42) || max_hits < 0)
    return fail(h, HG_ERR_ARGS, "hg_reserve: bad sizes (N %d, dim %d, max_hits %d)", max_N, dim, max_hits);
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, HG_ERR_CUDA, "cudaSetDevice");
  const long long bytes = refine_area_bytes(max_N, dim, max_hits);
  if (bytes > h->refine_pool_max) return HG_OK;  // such calls refine inline and use no pool
  return grow(h, &h->scratch, &h->scratch_bytes, bytes, false, "refinement scratch");
}

const char* hg_last_error_string(hg_handle* h) { return h ? h->err : "null handle"; }

int hg_propagate_fixed(hg_handle* h, double mu, int order, int dim, int N, const double* y0, long long ld_in,
                       const double* t_vals, int n_nodes, int out_every, double* y_out, long long ld_out, int fwd,
                       int flip_lo, int flip_hi, int* status, void* stream) {
  if (!h) return HG_ERR_ARGS;
  hg::FixedParams p;
  const int rc = fixed_common(h, mu, order, dim, N, y0, ld_in, t_vals, n_nodes, out_every, y_out, ld_out, fwd, flip_lo,
                              flip_hi, status, p);
  if (rc != HG_OK) return rc;
  return fixed_dispatch(h, order, dim, p, (cudaStream_t)stream);
}

int hg_propagate_fixed_event(hg_handle* h, double mu, int order, int dim, int N, const double* y0, long long ld_in,
                             const double* t_vals, int n_nodes, int out_every, double* y_out, long long ld_out,
                             int fwd, int flip_lo, int flip_hi, const hg_event* ev, double* hit_t, double* hit_y,
                             int* n_hits, int* status, void* stream) {
  if (!h) return HG_ERR_ARGS;
  hg::FixedParams p;
  const int rc = fixed_common(h, mu, order, dim, N, y0, ld_in, t_vals, n_nodes, out_every, y_out, ld_out, fwd, flip_lo,
                              flip_hi, status, p);
  if (rc != HG_OK) return rc;
  if (!ev || ev->index < 0 || ev->index >= dim) return fail(h, HG_ERR_ARGS, "event index out of range");
  if (ev->direction < -1 || ev->direction > 1) return fail(h, HG_ERR_ARGS, "bad event direction");
  if (N > 0 && (!hit_t || !hit_y || !n_hits)) return fail(h, HG_ERR_ARGS, "hit buffers are null");
  p.ev_index = ev->index;
  p.ev_offset = ev->offset;
  p.ev_dir = ev->direction;
  p.xtol = ev->xtol;
  p.gtol = ev->gtol;
  p.hit_t = hit_t;
  p.hit_y = hit_y;
  p.n_hits = n_hits;
  return fixed_dispatch(h, order, dim, p, (cudaStream_t)stream);
}

}  // extern "C"

// Argument checks and kernel parameters shared by the DOP853 entry points.
static int dop853_setup(hg_handle* h, double mu, int dim, int N, const double* y0, long long ld,
                        const double* t0_arr, const double* tmax_arr, double t0, double tmax,
                        const hg_dop853_opts* opts, const hg_event* ev, int n_samples, int sample_last_only,
                        double* y_samples, double* y_end, double* t_end, double* hit_t, double* hit_y, int* n_hits,
                        int* n_accept, int* n_reject, int* status, hg::DopParams& p) {
  if (dim != 6 && dim != 42) return fail(h, HG_ERR_ARGS, "dim must be 6 or 42 (got %d)", dim);
  if (N < 0 || ld < N) return fail(h, HG_ERR_ARGS, "bad N/ld");
  if (!opts) return fail(h, HG_ERR_ARGS, "opts is null");
  if (N > 0 && !y0) return fail(h, HG_ERR_ARGS, "y0 is null");
  if (opts->flip_lo < 0 || opts->flip_hi > dim || opts->flip_lo > opts->flip_hi)
    return fail(h, HG_ERR_ARGS, "bad flip range");
  if (!(opts->rtol >= 0.0) || !(opts->atol >= 0.0)) return fail(h, HG_ERR_ARGS, "negative tolerance");
  if (!(opts->min_step > 0.0) || !(opts->max_step > 0.0)) return fail(h, HG_ERR_ARGS, "step bounds must be > 0");
  if (opts->max_steps < 1) return fail(h, HG_ERR_ARGS, "max_steps must be >= 1");
  if (n_samples < 0 || n_samples == 1) return fail(h, HG_ERR_ARGS, "n_samples must be 0 or >= 2");
  if (n_samples >= 2 && !y_samples) return fail(h, HG_ERR_ARGS, "y_samples is null");
  memset(&p, 0, sizeof(p));
  p.ev_index = -1;
  if (ev && ev->index >= 0) {
    if (ev->index >= dim) return fail(h, HG_ERR_ARGS, "event index out of range");
    if (ev->max_hits < 1) return fail(h, HG_ERR_ARGS, "max_hits must be >= 1");
    if (ev->direction < -1 || ev->direction > 1) return fail(h, HG_ERR_ARGS, "bad event direction");
    if (!hit_t || !hit_y) return fail(h, HG_ERR_ARGS, "hit buffers are null");
    p.ev_index = ev->index;
    p.ev_offset = ev->offset;
    p.ev_dir = ev->direction;
    p.max_hits = ev->max_hits;
    p.xtol = ev->xtol;
    p.gtol = ev->gtol;
  }
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, HG_ERR_CUDA, "cudaSetDevice");
  p.N = N;
  p.mu = mu;
  p.dir = make_dir(dim, opts->fwd, opts->flip_lo, opts->flip_hi);
  p.y0 = y0;
  p.ld = ld;
  p.t0_arr = t0_arr;
  p.tmax_arr = tmax_arr;
  p.t0 = t0;
  p.tmax = tmax;
  p.rtol = opts->rtol;
  p.atol = opts->atol;
  p.max_step = opts->max_step;
  p.min_step = opts->min_step;
  p.max_steps = opts->max_steps;
  p.m = n_samples;
  p.dense_last = sample_last_only ? 1 : 0;
  p.y_out = y_samples;
  p.y_end = y_end;
  p.t_end = t_end;
  p.hit_t = hit_t;
  p.hit_y = hit_y;
  p.n_hits = n_hits;
  p.n_accept = n_accept;
  p.n_reject = n_reject;
  p.status = status;
  return HG_OK;
}

extern "C" {

int hg_propagate_dop853(hg_handle* h, double mu, int dim, int N, const double* y0, long long ld,
                        const double* t0_arr, const double* tmax_arr, double t0, double tmax,
                        const hg_dop853_opts* opts, const hg_event* ev, int n_samples, int sample_last_only,
                        double* y_samples, double* y_end, double* t_end, double* hit_t, double* hit_y, int* n_hits,
                        int* n_accept, int* n_reject, int* status, void* stream) {
  if (!h) return HG_ERR_ARGS;
  hg::DopParams p;
  const int rc = dop853_setup(h, mu, dim, N, y0, ld, t0_arr, tmax_arr, t0, tmax, opts, ev, n_samples,
                              sample_last_only, y_samples, y_end, t_end, hit_t, hit_y, n_hits, n_accept, n_reject,
                              status, p);
  if (rc != HG_OK || N == 0) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // crossings are refined after the integration through a record pool, or
  // inline (same bits) when the pool would exceed refine_pool_max
  if (defer_refine(p) && refine_area_bytes(N, dim, p.max_hits) <= h->refine_pool_max) {
    int e = ensure_scratch(h, refine_area_bytes(N, dim, p.max_hits));
    if (e != HG_OK) return e;
    refine_area_carve(N, p.max_hits, h->scratch, p);
    if (cudaMemsetAsync(p.refine_count, 0, sizeof(int), s) != cudaSuccess) return fail(h, HG_ERR_CUDA, "memset");
  }
  int rc2;
  if (dim == 6) {
    int lanes = h->lanes_d6;
    if (lanes == 0) lanes = auto_lanes_d6(h, N);
    if (lanes == 6)
      rc2 = launch_dop853<6>(h, p, s);
    else if (lanes == 2)
      rc2 = launch_dop853<2>(h, p, s);
    else
      rc2 = launch_dop853<1>(h, p, s);
  } else {
    const int g = p.ev_index < 0 ? lanes_d42_dop_free(h, N) : lanes_d42(h, N);
    if (g == 12 && p.ev_index < 0)
      rc2 = launch_dop853_pair(h, p, s);
    else if (g == 18 && p.ev_index < 0)
      rc2 = launch_dop853_trio(h, p, s);
    else
      rc2 = g == 14 ? launch_dop853<14>(h, p, s) : launch_dop853<7>(h, p, s);
  }
  if (rc2 != HG_OK) return rc2;
  return refine_pending(h, p, dim, s);
}

long long hg_dop853_segmented_workspace_bytes(int N, int dim, int max_hits) {
  if (N < 0 || (dim != 6 && dim != 42) || max_hits < 0) return -1;
  return seg_ws_layout(N, dim, max_hits, nullptr, nullptr);
}

int hg_propagate_dop853_segmented(hg_handle* h, double mu, int dim, int N, const double* y0, long long ld,
                                  const double* t0_arr, const double* tmax_arr, double t0, double tmax,
                                  const hg_dop853_opts* opts, const hg_event* ev, int n_samples,
                                  int sample_last_only, double* y_samples, double* y_end, double* t_end,
                                  double* hit_t, double* hit_y, int* n_hits, int* n_accept, int* n_reject,
                                  int* status, int seg_steps, int max_segments, int resume, void* workspace,
                                  long long workspace_bytes, void* stream) {
  if (!h) return HG_ERR_ARGS;
  if (seg_steps < 1 || max_segments < 1) return fail(h, HG_ERR_ARGS, "seg_steps and max_segments must be >= 1");
  if (N > 0 && (!y_end || !t_end || !n_accept || !n_reject || !status))
    return fail(h, HG_ERR_ARGS, "segmented runs keep their state in y_end/t_end/n_accept/n_reject/status");
  if (ev && ev->index >= 0 && N > 0 && !n_hits) return fail(h, HG_ERR_ARGS, "n_hits is required with an event");
  const int ws_hits = (ev && ev->index >= 0 && ev->max_hits > 0) ? ev->max_hits : 0;
  if (!workspace || workspace_bytes < seg_ws_layout(N, dim, ws_hits, nullptr, nullptr))
    return fail(h, HG_ERR_ARGS, "workspace smaller than hg_dop853_segmented_workspace_bytes(N, dim, max_hits)");
  // argument checks and parameter setup shared with the single-pass entry
  hg::DopParams p;
  memset(&p, 0, sizeof(p));
  int rc = dop853_setup(h, mu, dim, N, y0, ld, t0_arr, tmax_arr, t0, tmax, opts, ev, n_samples, sample_last_only,
                        y_samples, y_end, t_end, hit_t, hit_y, n_hits, n_accept, n_reject, status, p);
  if (rc != HG_OK || N == 0) return rc;
  SegWs w;
  seg_ws_layout(N, dim, ws_hits, (char*)workspace, &w);
  cudaStream_t s = (cudaStream_t)stream;
  // crossings of this call are refined at its end
  if (defer_refine(p)) {
    refine_area_carve(N, p.max_hits, w.refine, p);
    if (cudaMemsetAsync(p.refine_count, 0, sizeof(int), s) != cudaSuccess) return fail(h, HG_ERR_CUDA, "memset");
  }
  if (dim == 6) {
    int lanes = h->lanes_d6;
    if (lanes == 0) lanes = auto_lanes_d6(h, N);
    if (lanes == 6)
      rc = launch_dop853_seg<6>(h, p, w, seg_steps, max_segments, resume, s);
    else if (lanes == 2)
      rc = launch_dop853_seg<2>(h, p, w, seg_steps, max_segments, resume, s);
    else
      rc = launch_dop853_seg<1>(h, p, w, seg_steps, max_segments, resume, s);
  } else {
    rc = lanes_d42(h, N) == 14 ? launch_dop853_seg<14>(h, p, w, seg_steps, max_segments, resume, s)
                               : launch_dop853_seg<7>(h, p, w, seg_steps, max_segments, resume, s);
  }
  if (rc != HG_OK) return rc;
  return refine_pending(h, p, dim, s);
}

int hg_propagate_dop853_scheduled(hg_handle* h, double mu, int dim, int N, const double* y0, long long ld,
                                  const double* t0_arr, const double* tmax_arr, double t0, double tmax,
                                  const hg_dop853_opts* opts, const hg_event* ev, int n_samples,
                                  int sample_last_only, double* y_samples, double* y_end, double* t_end,
                                  double* hit_t, double* hit_y, int* n_hits, int* n_accept, int* n_reject,
                                  int* status, void* workspace, long long workspace_bytes, void* stream) {
  if (!h) return HG_ERR_ARGS;
  if (N > 0 && (!y_end || !t_end || !n_accept || !n_reject || !status))
    return fail(h, HG_ERR_ARGS, "scheduled runs keep their state in y_end/t_end/n_accept/n_reject/status");
  if (ev && ev->index >= 0 && N > 0 && !n_hits) return fail(h, HG_ERR_ARGS, "n_hits is required with an event");
  const int ws_hits = (ev && ev->index >= 0 && ev->max_hits > 0) ? ev->max_hits : 0;
  if (!workspace || workspace_bytes < seg_ws_layout(N, dim, ws_hits, nullptr, nullptr))
    return fail(h, HG_ERR_ARGS, "workspace smaller than hg_dop853_segmented_workspace_bytes(N, dim, max_hits)");
  hg::DopParams p;
  memset(&p, 0, sizeof(p));
  int rc = dop853_setup(h, mu, dim, N, y0, ld, t0_arr, tmax_arr, t0, tmax, opts, ev, n_samples, sample_last_only,
                        y_samples, y_end, t_end, hit_t, hit_y, n_hits, n_accept, n_reject, status, p);
  if (rc != HG_OK || N == 0) return rc;
  SegWs w;
  seg_ws_layout(N, dim, ws_hits, (char*)workspace, &w);
  cudaStream_t s = (cudaStream_t)stream;
  if (defer_refine(p)) {
    refine_area_carve(N, p.max_hits, w.refine, p);
    if (cudaMemsetAsync(p.refine_count, 0, sizeof(int), s) != cudaSuccess) return fail(h, HG_ERR_CUDA, "memset");
  }
  rc = seg_init(h, p, w, s);
  if (rc != HG_OK) return rc;
  // every segment finishes its trajectories or advances each by seg_steps
  // attempted steps, and no trajectory exceeds max_steps: this bounds the loop
  const long long seg = h->seg_steps;
  const long long max_iter = p.max_steps / seg + 2;
  int n_live = N, a = 0;
  for (long long it = 0; it < max_iter && n_live > 0; ++it) {
    if (dim == 6) {
      const int g = sched_lanes_d6(h, n_live);
      if (g == 6)
        rc = launch_segment<6>(h, p, w, (int)seg, a, n_live, s);
      else if (g == 2)
        rc = launch_segment<2>(h, p, w, (int)seg, a, n_live, s);
      else
        rc = launch_segment<1>(h, p, w, (int)seg, a, n_live, s);
    } else if (lanes_d42(h, n_live) == 14) {
      rc = launch_segment<14>(h, p, w, (int)seg, a, n_live, s);
    } else {
      rc = launch_segment<7>(h, p, w, (int)seg, a, n_live, s);
    }
    if (rc != HG_OK) return rc;
    a ^= 1;
    cudaError_t e = cudaMemcpyAsync(h->host_count, w.count + a, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(h, HG_ERR_CUDA, "segment: %s", cudaGetErrorString(e));
    n_live = *h->host_count;
  }
  if (n_live > 0) return fail(h, HG_ERR_CUDA, "scheduled DOP853 did not finish within its step bound");
  rc = refine_pending(h, p, dim, s);
  if (rc != HG_OK) return rc;
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(h, HG_ERR_CUDA, "refine: %s", cudaGetErrorString(e));
  return HG_OK;
}

int hg_set_tuning(hg_handle* h, int key, int value) {
  if (!h) return HG_ERR_ARGS;
  switch (key) {
    case HG_TUNE_BLOCK_THREADS:
      if (value != 32 && value != 64 && value != 128) return fail(h, HG_ERR_ARGS, "block must be 32, 64 or 128");
      h->block = value;
      return HG_OK;
    case HG_TUNE_DOP853_LANES_D6:
      if (value != 0 && value != 1 && value != 2 && value != 6)
        return fail(h, HG_ERR_ARGS, "lanes must be 0 (auto), 1, 2 or 6");
      h->lanes_d6 = value;
      return HG_OK;
    case HG_TUNE_REFINE_POOL_MB:
      if (value < 0) return fail(h, HG_ERR_ARGS, "pool size must be >= 0 MB");
      h->refine_pool_max = (long long)value << 20;
      return HG_OK;
    case HG_TUNE_SM_CAPACITY:
      if (value < 5 || value > 640) return fail(h, HG_ERR_ARGS, "capacity (tenths of warps per SM) must be in [5, 640]");
      h->sm_capacity_x10 = value;
      return HG_OK;
    case HG_TUNE_LANES_D42:
      if (value != 0 && value != 7 && value != 14 && value != 12 && value != 18)
        return fail(h, HG_ERR_ARGS, "lanes must be 0 (auto), 7, 14, 12 (paired warps) or 18 (three warps)");
      h->lanes_d42 = value;
      return HG_OK;
    case HG_TUNE_SPREAD:
      if (value != 0 && value != 1) return fail(h, HG_ERR_ARGS, "spread must be 0 or 1");
      h->spread = value;
      return HG_OK;
    case HG_TUNE_SEG_STEPS:
      if (value < 1 || value > 1000000) return fail(h, HG_ERR_ARGS, "segment steps must be in [1, 1e6]");
      h->seg_steps = value;
      return HG_OK;
    default:
      return fail(h, HG_ERR_ARGS, "unknown tuning key %d", key);
  }
}

int hg_get_counter(hg_handle* h, int key, long long* value) {
  if (!h || !value) return HG_ERR_ARGS;
  if (key == HG_COUNTER_KERNEL_LAUNCHES) *value = h->launches;
  else if (key == HG_COUNTER_ALLOCATIONS) *value = h->allocs;
  else return fail(h, HG_ERR_ARGS, "unknown counter %d", key);
  return HG_OK;
}

int hg_get_tuning(hg_handle* h, int key, int* value) {
  if (!h || !value) return HG_ERR_ARGS;
  if (key == HG_TUNE_BLOCK_THREADS) *value = h->block;
  else if (key == HG_TUNE_DOP853_LANES_D6) *value = h->lanes_d6;
  else if (key == HG_TUNE_SEG_STEPS) *value = h->seg_steps;
  else if (key == HG_TUNE_SPREAD) *value = h->spread;
  else if (key == HG_TUNE_LANES_D42) *value = h->lanes_d42;
  else if (key == HG_TUNE_SM_CAPACITY) *value = h->sm_capacity_x10;
  else if (key == HG_TUNE_REFINE_POOL_MB) *value = (int)(h->refine_pool_max >> 20);
  else return fail(h, HG_ERR_ARGS, "unknown tuning key %d", key);
  return HG_OK;
}

int hg_selftest_bounded_wait(hg_handle* h, int limit_ms, int* out3, void* stream) {
  if (!h || !out3 || limit_ms < 1 || limit_ms > 2000) return fail(h, HG_ERR_ARGS, "bad self-test arguments");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, HG_ERR_CUDA, "cudaSetDevice");
  hg::bounded_wait_selftest_kernel<<<1, 64, 0, (cudaStream_t)stream>>>(out3, 1000000ull * (unsigned long long)limit_ms);
  return check_launch(h, "bounded_wait_selftest_kernel");
}

int hg_probe_fp64_peak(hg_handle* h, double* tflops) {
  if (!h || !tflops) return HG_ERR_ARGS;
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, HG_ERR_CUDA, "cudaSetDevice");
  double* out = reinterpret_cast<double*>(h->counters);  // never written in practice
  const int threads = 256, blocks = h->sm_count * 8, iters = 4096;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fp64_probe_kernel<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(a);
  fp64_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(b);
  const cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return fail(h, HG_ERR_CUDA, "probe: %s", cudaGetErrorString(e));
  const double flops = 2.0 * 8.0 * (double)iters * threads * (double)blocks;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return HG_OK;
}

}  // extern "C"

// Library-internal access to the handle for the other translation units
// (hg_internal.h): not part of the C ABI.
namespace hg_internal {

int correct_buffers(hg_handle* h, long long bytes, void** out) {
  *out = nullptr;
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, HG_ERR_CUDA, "cudaSetDevice");
  const int rc = grow(h, &h->corr, &h->corr_bytes, bytes, false, "corrector buffers");
  *out = rc == HG_OK ? h->corr : nullptr;
  return rc;
}

int reserve_refine(hg_handle* h, int N, int dim, int max_hits) { return hg_reserve(h, N, dim, max_hits); }

int fail_msg(hg_handle* h, int code, const char* msg) { return fail(h, code, "%s", msg); }

void** graph_slot(hg_handle* h, void (*free_fn)(void*)) {
  h->corr_graph_free = free_fn;
  return &h->corr_graph;
}

void count_launches(hg_handle* h, long long n) { h->launches += n; }

int device_of(const hg_handle* h) { return h->device; }

int tuning(const hg_handle* h, int key) {
  if (key == HG_TUNE_DOP853_LANES_D6) return h->lanes_d6;
  if (key == HG_TUNE_LANES_D42) return h->lanes_d42;
  if (key == HG_TUNE_BLOCK_THREADS) return h->block;
  return 0;
}

}  // namespace hg_internal
