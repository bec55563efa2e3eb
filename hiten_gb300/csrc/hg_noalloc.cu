// hg_propagate_dop853_noalloc: the adaptive DOP853 propagation of
// hg_propagate_dop853 for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or forbidden
// -- a host that hands us only pre-allocated buffers (an embedding runtime
// with its own memory pool, a real-time loop that must not allocate after
// start-up, a plugin that is not allowed to create a library handle).  The
// ordinary entry points allocate their scratch once, in hg_create; this one
// needs no handle and allocates nothing, ever.
//
// The only scratch the kernel needs beyond the caller's inputs and outputs is
// the lane-refill counter (a 32-bit int that finished lanes increment to claim
// the next trajectory).  It lives in the file-scope device array below,
// HG_NOALLOC_SCRATCH_BYTES (256 bytes) per device, which every GPU that loads
// the library holds until the process exits.  Host code may not pass the
// array's name to a kernel (on the host it is only a stand-in symbol, not a
// device address), so the first call on each device resolves the real
// device address with cudaGetSymbolAddress, with that device current, and
// caches it.  Make that first call before any stream capture begins.  The
// cached address is tagged with the CUDA context it was resolved in; when the
// current context differs (after cudaDeviceReset, the module and its array
// are loaded again, possibly elsewhere) the next call resolves it again
// before any device work, so a reset never leaves a stale address behind.
//
// All calls share the one counter: it is cleared (cudaMemsetAsync on the
// caller's stream) at the start of every call, so calls that overlap on the
// GPU -- on different streams, or from different host threads -- race on it
// and must be serialized by the caller.  N is limited to HG_NOALLOC_MAX_N so
// that the 32-bit counter cannot overflow.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "hg_kernels.cuh"
#include "hitengpu.h"

namespace {

constexpr int kMaxDevices = 64;
constexpr int kBlock = 32;  // one warp per block: spreads small batches over all 152 SMs

static __device__ __align__(256) int hg_noalloc_scratch[HG_NOALLOC_SCRATCH_BYTES / sizeof(int)];

std::mutex g_setup_mutex;
struct ScratchEntry {
  int* ptr = nullptr;
  unsigned long long ctx_id = 0;  // context the address was resolved in
};
ScratchEntry g_scratch[kMaxDevices];

// Identity of the calling thread's current CUDA context (driver entry points
// looked up through the runtime, so the library needs no link to libcuda); 0
// when no context is current yet or the driver lacks cuCtxGetId.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)f;
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the scratch array on `device` (the current device),
// resolved once per context.
int scratch_address(int device, int** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  ScratchEntry& e = g_scratch[device];
  const unsigned long long id = current_context_id();
  if (!e.ptr || id == 0 || id != e.ctx_id) {
    int* ptr = nullptr;
    const cudaError_t err = cudaGetSymbolAddress((void**)&ptr, hg_noalloc_scratch);
    if (err != cudaSuccess || !ptr) return HG_ERR_CUDA;
    e.ptr = ptr;
    e.ctx_id = current_context_id();  // the lookup made the device's context current
  }
  *out = e.ptr;
  return HG_OK;
}

template <int G>
int launch(hg::DopParams p, int device, int* counter, cudaStream_t s) {
  int sm_count = 0;
  if (cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return HG_ERR_CUDA;
  // launches without dense samples run the kernel built without that path
  // (fewer registers), as the handle entry point does
  auto kern = p.m >= 2 ? hg::dop853_kernel<G, true> : hg::dop853_kernel<G, false>;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  const int tpb = (kBlock / 32) * hg::Layout<G>::TPW;
  const int need = (p.N + tpb - 1) / tpb;
  const int cap = per_sm * sm_count;
  const int grid = need < cap ? need : cap;
  p.stride = grid * tpb;
  p.next_traj = nullptr;
  if (need > cap) {
    if (cudaMemsetAsync(counter, 0, sizeof(int), s) != cudaSuccess) return HG_ERR_CUDA;
    p.next_traj = counter;
  }
  kern<<<grid, kBlock, 0, s>>>(p);
  return cudaGetLastError() == cudaSuccess ? HG_OK : HG_ERR_CUDA;
}

}  // namespace

extern "C" int hg_propagate_dop853_noalloc(double mu, int dim, int N, const double* y0, long long ld,
                                           const double* t0_arr, const double* tmax_arr, double t0, double tmax,
                                           const hg_dop853_opts* opts, const hg_event* ev, int n_samples,
                                           int sample_last_only, double* y_samples, double* y_end, double* t_end,
                                           double* hit_t, double* hit_y, int* n_hits, int* n_accept, int* n_reject,
                                           int* status, void* stream) {
  if (dim != 6 && dim != 42) return HG_ERR_ARGS;
  if (N < 0 || N > HG_NOALLOC_MAX_N || ld < N) return HG_ERR_ARGS;
  if (!opts || (N > 0 && !y0)) return HG_ERR_ARGS;
  if (opts->flip_lo < 0 || opts->flip_hi > dim || opts->flip_lo > opts->flip_hi) return HG_ERR_ARGS;
  if (!(opts->rtol >= 0.0) || !(opts->atol >= 0.0) || !(opts->min_step > 0.0) || !(opts->max_step > 0.0) ||
      opts->max_steps < 1)
    return HG_ERR_ARGS;
  if (n_samples < 0 || n_samples == 1 || (n_samples >= 2 && !y_samples)) return HG_ERR_ARGS;
  hg::DopParams p;
  memset(&p, 0, sizeof(p));
  p.ev_index = -1;
  if (ev && ev->index >= 0) {
    if (ev->index >= dim || ev->max_hits < 1 || ev->direction < -1 || ev->direction > 1 || !hit_t || !hit_y)
      return HG_ERR_ARGS;
    p.ev_index = ev->index;
    p.ev_offset = ev->offset;
    p.ev_dir = ev->direction;
    p.max_hits = ev->max_hits;
    p.xtol = ev->xtol;
    p.gtol = ev->gtol;
  }
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return HG_ERR_NO_DEVICE;
  int* counter = nullptr;
  if (scratch_address(device, &counter) != HG_OK) return HG_ERR_CUDA;
  if (N == 0) return HG_OK;
  p.N = N;
  p.mu = mu;
  p.dir.neg_lo = opts->fwd == -1 ? opts->flip_lo : 0;
  p.dir.neg_hi = opts->fwd == -1 ? opts->flip_hi : 0;
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
  cudaStream_t s = (cudaStream_t)stream;
  if (dim == 6) return launch<1>(p, device, counter, s);
  return launch<7>(p, device, counter, s);
}
