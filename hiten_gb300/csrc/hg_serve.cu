// Native request server for DOP853 propagation requests: continuous batching
// at the level of trajectory slots.
//
// Every problem (mu, dim, span, options, event) that has work gets a pool of
// C trajectory slots resident on the device: the states, step sizes,
// controller memory, counters and crossings of every live trajectory stay in
// the pool between segments.  A pool's thread loops:
//   1. admission: trajectories of waiting requests of its problem take free
//      slots (a request can enter over several rounds; its inputs are copied
//      through pinned staging and scattered into the slots by a kernel);
//   2. one segment: every live slot advances by up to seg_steps attempted
//      steps (the library's DOP853 kernel in list mode; its lane layout chosen
//      from the live count, as the scheduled driver does), then the saved
//      crossings are refined;
//   3. collection: a kernel gathers the result rows of the slots that
//      finished straight into pinned host staging (mapped into the device's
//      address space; two halves used in turn), the live and finished counts
//      follow in one 16-byte copy, and the thread synchronizes once per
//      segment.  The finished slots are free for the next admission at once;
//      their rows are copied into the requests while the next segment runs.
// So a request arriving while others run is admitted at the next segment
// boundary as slots free up, and its work overlaps theirs on the device.
// Trajectories never interact and a paused trajectory resumes with every
// bit, so each request's results equal a direct hg_propagate_dop853 call on
// it alone.
//
// Memory: hg_serve_create allocates a device arena of hbm_budget_bytes and a
// pinned host arena of staging_bytes; a pool takes one block of each when it
// opens (its slot count C = pool_slots, halved until the free arenas hold it)
// and returns them when its problem has no work left.  Nothing is allocated
// after creation.
#include <cuda_runtime.h>
#include <limits.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "hg_kernels.cuh"
#include "hitengpu.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Key {
  double mu, t0, tmax;
  int dim;
  hg_dop853_opts o;
  int has_ev;
  hg_event ev;
};

bool same_key(const Key& a, const Key& b) { return memcmp(&a, &b, sizeof(Key)) == 0; }

struct Request {
  long long id;
  Key key;
  int n;
  std::vector<double> y0;  // row-major (n, dim)
  int admitted = 0;        // trajectories given a slot so far
  int done = 0;            // trajectories finished
  // results (row-major)
  std::vector<double> y_end, t_end, hit_t, hit_y;
  std::vector<int> n_hits, n_acc, n_rej, status;
  int state = 0;  // 0 pending, 1 running, 2 done, 3 failed
  int error = HG_OK;
  Clock::time_point submitted, finished;
};

// First-fit allocator over one fixed block of memory (offsets only).
class Arena {
 public:
  void reset(long long size) {
    free_.clear();
    if (size > 0) free_[0] = size;
  }
  long long alloc(long long bytes) {
    bytes = up(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        const long long off = it->first, len = it->second;
        free_.erase(it);
        if (len > bytes) free_[off + bytes] = len - bytes;
        return off;
      }
    }
    return -1;
  }
  void release(long long off, long long bytes) {
    bytes = up(bytes);
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  long long largest() const {
    long long m = 0;
    for (const auto& f : free_) m = std::max(m, f.second);
    return m;
  }
  static long long up(long long x) { return (x + 255) & ~255LL; }

 private:
  std::map<long long, long long> free_;  // offset -> length, disjoint, not adjacent
};

// Doubles and ints of one finished trajectory's result row.
struct RowShape {
  int dim, hits;
  int nd() const { return dim + 1 + hits + hits * dim; }  // y_end, t_end, hit_t, hit_y
  static constexpr int ni = 4;                            // n_accept, n_reject, n_hits, status
};

// A pool's device and staging layout for C slots.
struct PoolLayout {
  long long dev_bytes = 0, stg_bytes = 0;
  // device offsets
  long long y0, y_end, t_end, hit_t, hit_y, wh, wep, wpp, wq, na, nr, nh, st, list0, list1, cnt, stage_y0,
      stage_slots, refine;
  // staging offsets (pinned): admission inputs, then two halves of counts and
  // finished rows (a segment's collection writes one while the rows of the
  // segment before are delivered from the other)
  long long s_y0, s_slots, s_cnt[2], s_fin[2], s_out_d[2], s_out_i[2];
  PoolLayout(int C, int dim, int hits) {
    const RowShape rs{dim, hits};
    const long long c = C;
    auto D = [&](long long& o, long long bytes) {
      o = dev_bytes;
      dev_bytes += Arena::up(bytes);
    };
    D(y0, 8 * dim * c);
    D(y_end, 8 * dim * c);
    D(t_end, 8 * c);
    D(hit_t, 8 * hits * c + 8);
    D(hit_y, 8 * hits * dim * c + 8);
    D(wh, 8 * c);
    D(wep, 8 * c);
    D(wpp, 8 * c);
    D(wq, 4 * c);
    D(na, 4 * c);
    D(nr, 4 * c);
    D(nh, 4 * c);
    D(st, 4 * c);
    D(list0, 4 * c);
    D(list1, 4 * c);
    D(cnt, 64);
    D(stage_y0, 8 * dim * c);
    D(stage_slots, 4 * c);
    const long long recs = c * std::max(hits, 1);
    D(refine, hits > 0 ? 256 + 2 * Arena::up(recs * 4) + Arena::up((15LL * dim + 3) * recs * 8) : 256);
    auto S = [&](long long& o, long long bytes) {
      o = stg_bytes;
      stg_bytes += Arena::up(bytes);
    };
    S(s_y0, 8 * dim * c);
    S(s_slots, 4 * c);
    for (int h = 0; h < 2; ++h) {
      S(s_cnt[h], 64);
      S(s_fin[h], 4 * c);
      S(s_out_d[h], 8LL * rs.nd() * c);
      S(s_out_i[h], 4LL * RowShape::ni * c);
    }
  }
};

// New trajectories into their slots: inputs, "not started" status, the tail
// of the live list; the live count becomes live + n.
__global__ void admit_kernel(int n, int C, int dim, const double* stage, const int* slots, double* y0, int* status,
                             int* list, int* count, int live) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int s = slots[j];
    for (int c = 0; c < dim; ++c) y0[(long long)c * C + s] = stage[(long long)c * n + j];
    status[s] = -2;
    list[live + j] = s;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = live + n;
}

// Slots of the last segment's list that finished: their result rows,
// gathered (fin[k] = slot of row k; *n_fin rows).  fin, out_d and out_i are
// the device addresses of pinned host staging.
__global__ void collect_kernel(int C, int dim, int hits, const int* list, const int* n_in, const double* y_end,
                               const double* t_end, const double* hit_t, const double* hit_y, const int* na,
                               const int* nr, const int* nh, const int* st, int* fin, int* n_fin, double* out_d,
                               int* out_i) {
  const int n = *n_in;
  const int nd = dim + 1 + hits + hits * dim;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int s = list[j];
    if (st[s] == HG_RUNNING) continue;
    const int k = atomicAdd(n_fin, 1);
    fin[k] = s;
    double* r = out_d + (long long)k * nd;
    for (int c = 0; c < dim; ++c) r[c] = y_end[(long long)c * C + s];
    r[dim] = t_end[s];
    const int h = hits ? nh[s] : 0;
    for (int q = 0; q < hits; ++q) {
      r[dim + 1 + q] = q < h ? hit_t[(long long)q * C + s] : 0.0;
      for (int c = 0; c < dim; ++c)
        r[dim + 1 + hits + q * dim + c] = q < h ? hit_y[((long long)q * dim + c) * C + s] : 0.0;
    }
    int* ri = out_i + (long long)k * RowShape::ni;
    ri[0] = na[s];
    ri[1] = nr[s];
    ri[2] = h;
    ri[3] = st[s];
  }
}

template <class K>
int resident_blocks(K kern, int block, int sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return per_sm * sms;
}

// One segment over the live list (its first `live` entries) in layout G.
template <int G>
cudaError_t segment(hg::DopParams p, int live, int sms, cudaStream_t s) {
  const int tpb = hg::Layout<G>::TPW;
  const int need = (live + tpb - 1) / tpb;
  const int cap = resident_blocks(hg::dop853_kernel<G, false>, 32, sms);
  const int grid = need < cap ? need : cap;
  if (grid < 1) return cudaSuccess;
  p.stride = grid * tpb;
  hg::dop853_kernel<G, false><<<grid, 32, 0, s>>>(p);
  return cudaGetLastError();
}

// The crossings the segment saved (records [0, *refine_count)).
template <int G>
cudaError_t refine(hg::DopParams p, int sms, cudaStream_t s) {
  const int tpb = hg::Layout<G>::TPW;
  const long long need = (p.rec_ld + tpb - 1) / tpb;
  const int cap = resident_blocks(hg::refine_kernel<G>, 32, sms);
  const int grid = need < cap ? (int)need : cap;
  if (grid < 1) return cudaSuccess;
  p.stride = grid * tpb;
  hg::refine_kernel<G><<<grid, 32, 0, s>>>(p);
  return cudaGetLastError();
}

// Lanes per trajectory for a segment of n live trajectories: the least
// lat(G) x max(1, warps / capacity), the host-scheduled driver's rule.
int lanes_for(int dim, int n, int sms) {
  const double cap = 3.0 * sms;
  if (dim == 6) {
    const int gs[3] = {1, 2, 6}, tpw[3] = {32, 16, 5};
    const double lat[3] = {1.0, 0.622, 0.400};
    int best = 0;
    double bc = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double warps = (double)((n + tpw[i] - 1) / tpw[i]);
      const double c = lat[i] * std::max(1.0, warps / cap);
      if (i == 0 || c < bc) {
        best = i;
        bc = c;
      }
    }
    return gs[best];
  }
  const double w7 = (double)((n + 3) / 4), w14 = (double)((n + 1) / 2);
  const double c7 = std::max(1.0, w7 / cap), c14 = 0.65 * std::max(1.0, w14 / cap);
  return c14 < c7 ? 14 : 7;
}

struct Pool {
  Key key;
  int dim = 6, hits = 0, C = 0, slot = -1;
  long long dev_off = -1, dev_len = 0, stg_off = -1, stg_len = 0;
  std::vector<int> free_slots;
  std::vector<std::pair<std::shared_ptr<Request>, int>> owner;  // per slot: request, trajectory index
  // rows gathered from finished slots (slots already free), not yet copied
  // into their requests: request, trajectory index, in row order
  std::vector<std::pair<std::shared_ptr<Request>, int>> held;
  std::thread runner;
  std::atomic<int> finished{0};
  int rc = HG_OK;
};

}  // namespace

struct hg_server {
  hg_serve_config cfg;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<Request>> pending;  // requests with trajectories not yet admitted
  std::map<long long, std::shared_ptr<Request>> all;
  std::vector<std::unique_ptr<Pool>> pools;
  std::vector<cudaStream_t> streams;
  std::vector<char> slot_busy;
  long long next_id = 1;
  char* dev_base = nullptr;
  char* stg_base = nullptr;
  char* stg_dev = nullptr;  // the staging arena's device address (mapped pinned memory)
  Arena dev_arena, stg_arena;
  bool stop = false;
  std::thread worker;
  std::vector<double> latencies_ms;
  long long segments = 0;
  int sms = 1;

  // Admission for one pool (lock held): trajectories of waiting requests of
  // its problem, in arrival order, take free slots.
  void take_admissions(Pool& P, std::vector<int>& slots, std::vector<std::pair<std::shared_ptr<Request>, int>>& who) {
    for (auto it = pending.begin(); it != pending.end() && !P.free_slots.empty();) {
      auto r = *it;
      if (!same_key(r->key, P.key)) {
        ++it;
        continue;
      }
      while (r->admitted < r->n && !P.free_slots.empty()) {
        const int s = P.free_slots.back();
        P.free_slots.pop_back();
        slots.push_back(s);
        who.emplace_back(r, r->admitted);
        P.owner[s] = {r, r->admitted};
        ++r->admitted;
      }
      r->state = 1;
      if (r->admitted == r->n)
        it = pending.erase(it);
      else
        ++it;
    }
  }

  // The pool's loop (its own thread): admit, advance one segment, collect;
  // returns when its problem has no trajectory live or waiting.
  int run_pool(Pool& P) {
    const Key& k = P.key;
    const int d = P.dim, H = P.hits, C = P.C;
    const RowShape rs{d, H};
    const PoolLayout L(C, d, H);
    cudaStream_t s = streams[P.slot];
    if (cudaSetDevice(cfg.device) != cudaSuccess) return HG_ERR_CUDA;
    char* dv = dev_base + P.dev_off;
    char* sg = stg_base + P.stg_off;
    char* sd = stg_dev + P.stg_off;  // the same staging block, as the device addresses it
    double* y0 = (double*)(dv + L.y0);
    int* status = (int*)(dv + L.st);
    int* lists[2] = {(int*)(dv + L.list0), (int*)(dv + L.list1)};
    int* cnt = (int*)(dv + L.cnt);  // [0], [1] counts of the two live lists, [2] finished rows
    hg::DopParams p;
    memset(&p, 0, sizeof(p));
    p.N = C;
    p.mu = k.mu;
    p.dir.neg_lo = k.o.fwd == -1 ? k.o.flip_lo : 0;
    p.dir.neg_hi = k.o.fwd == -1 ? k.o.flip_hi : 0;
    p.y0 = y0;
    p.ld = C;
    p.t0 = k.t0;
    p.tmax = k.tmax;
    p.rtol = k.o.rtol;
    p.atol = k.o.atol;
    p.max_step = k.o.max_step;
    p.min_step = k.o.min_step;
    p.max_steps = k.o.max_steps;
    p.ev_index = -1;
    if (k.has_ev) {
      p.ev_index = k.ev.index;
      p.ev_offset = k.ev.offset;
      p.ev_dir = k.ev.direction;
      p.max_hits = k.ev.max_hits;
      p.xtol = k.ev.xtol;
      p.gtol = k.ev.gtol;
      const long long recs = (long long)C * H;
      char* ra = dv + L.refine;
      p.refine_count = (int*)ra;
      p.refine_list = (int*)(ra + 256);
      p.refine_hit = (int*)(ra + 256 + Arena::up(recs * 4));
      p.rec = (double*)(ra + 256 + 2 * Arena::up(recs * 4));
      p.rec_ld = recs;
      p.hit_t = (double*)(dv + L.hit_t);
      p.hit_y = (double*)(dv + L.hit_y);
      p.n_hits = (int*)(dv + L.nh);
    }
    p.y_end = (double*)(dv + L.y_end);
    p.t_end = (double*)(dv + L.t_end);
    p.n_accept = (int*)(dv + L.na);
    p.n_reject = (int*)(dv + L.nr);
    p.status = status;
    p.seg = 1;
    p.seg_steps = cfg.seg_steps;
    p.ws_h = (double*)(dv + L.wh);
    p.ws_err_prev = (double*)(dv + L.wep);
    p.ws_prev_pow = (double*)(dv + L.wpp);
    p.ws_q = (int*)(dv + L.wq);
    int live = 0, a = 0, h = 0;
    std::vector<int> slots;
    std::vector<std::pair<std::shared_ptr<Request>, int>> who;
    for (;;) {
      slots.clear();
      who.clear();
      {
        std::lock_guard<std::mutex> g(mu);
        take_admissions(P, slots, who);
      }
      const int n_new = (int)slots.size();
      const bool run_seg = live + n_new > 0;
      const int b = a ^ 1;
      if (n_new > 0) {
        double* stg_y0 = (double*)(sg + L.s_y0);
        int* stg_slots = (int*)(sg + L.s_slots);
        for (int j = 0; j < n_new; ++j) {
          const auto& w = who[j];
          for (int c = 0; c < d; ++c) stg_y0[(long long)c * n_new + j] = w.first->y0[(size_t)w.second * d + c];
          stg_slots[j] = slots[j];
        }
        if (cudaMemcpyAsync(dv + L.stage_y0, stg_y0, 8ull * d * n_new, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(dv + L.stage_slots, stg_slots, 4ull * n_new, cudaMemcpyHostToDevice, s) != cudaSuccess)
          return HG_ERR_CUDA;
        const int blocks = std::min((n_new + 255) / 256, 1024);
        admit_kernel<<<blocks, 256, 0, s>>>(n_new, C, d, (const double*)(dv + L.stage_y0),
                                            (const int*)(dv + L.stage_slots), y0, status, lists[a], cnt + a, live);
        if (cudaGetLastError() != cudaSuccess) return HG_ERR_CUDA;
        live += n_new;
      }
      if (run_seg) {
        // one segment over the live list, then the crossings it saved
        if (cudaMemsetAsync(cnt + b, 0, sizeof(int), s) != cudaSuccess ||
            cudaMemsetAsync(cnt + 2, 0, sizeof(int), s) != cudaSuccess)
          return HG_ERR_CUDA;
        if (k.has_ev && cudaMemsetAsync(p.refine_count, 0, sizeof(int), s) != cudaSuccess) return HG_ERR_CUDA;
        p.active_in = lists[a];
        p.n_in = cnt + a;
        p.active_out = lists[b];
        p.n_out = cnt + b;
        const int g = lanes_for(d, live, sms);
        cudaError_t e;
        if (d == 6)
          e = g == 6 ? segment<6>(p, live, sms, s)
                     : (g == 2 ? segment<2>(p, live, sms, s) : segment<1>(p, live, sms, s));
        else
          e = g == 14 ? segment<14>(p, live, sms, s) : segment<7>(p, live, sms, s);
        if (e == cudaSuccess && k.has_ev) e = d == 6 ? refine<1>(p, sms, s) : refine<7>(p, sms, s);
        if (e != cudaSuccess) return HG_ERR_CUDA;
        // finished slots of this segment's list: rows gathered into staging half h
        const int blocks = std::min((live + 255) / 256, 1024);
        collect_kernel<<<blocks, 256, 0, s>>>(C, d, H, lists[a], cnt + a, p.y_end, p.t_end, p.hit_t, p.hit_y,
                                              p.n_accept, p.n_reject, (const int*)(dv + L.nh), status,
                                              (int*)(sd + L.s_fin[h]), cnt + 2, (double*)(sd + L.s_out_d[h]),
                                              (int*)(sd + L.s_out_i[h]));
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(sg + L.s_cnt[h], cnt, 16, cudaMemcpyDeviceToHost, s) != cudaSuccess)
          return HG_ERR_CUDA;
      }
      // the rows of the segment before (staging half h ^ 1) go to their
      // requests while this one runs
      deliver(P, rs, (const double*)(sg + L.s_out_d[h ^ 1]), (const int*)(sg + L.s_out_i[h ^ 1]));
      if (!run_seg) return HG_OK;  // no trajectory live or waiting for this problem
      if (cudaStreamSynchronize(s) != cudaSuccess) return HG_ERR_CUDA;
      const int* sc = (const int*)(sg + L.s_cnt[h]);
      const int n_fin = sc[2];
      const int next_live = sc[b];
      {
        std::lock_guard<std::mutex> g(mu);
        ++segments;
        const int* fin = (const int*)(sg + L.s_fin[h]);
        for (int q = 0; q < n_fin; ++q) {
          const int sl = fin[q];
          P.held.push_back(std::move(P.owner[sl]));
          P.owner[sl] = {};
          P.free_slots.push_back(sl);
        }
      }
      live = next_live;
      a = b;
      h ^= 1;
    }
  }

  // Copies the held rows (in row order, from the staging half `od` / `oi`)
  // into their requests, then marks the requests they complete.  Only the
  // pool's thread writes a request's result arrays, and fetch reads them
  // only after the state turns 2 under the lock.
  void deliver(Pool& P, const RowShape& rs, const double* od, const int* oi) {
    if (P.held.empty()) return;
    const int d = rs.dim, H = rs.hits;
    for (size_t q = 0; q < P.held.size(); ++q) {
      Request& r = *P.held[q].first;
      const int i = P.held[q].second;
      const double* row = od + (long long)q * rs.nd();
      for (int c = 0; c < d; ++c) r.y_end[(size_t)i * d + c] = row[c];
      r.t_end[i] = row[d];
      for (int j = 0; j < H; ++j) {
        r.hit_t[(size_t)i * H + j] = row[d + 1 + j];
        for (int c = 0; c < d; ++c) r.hit_y[((size_t)i * H + j) * d + c] = row[d + 1 + H + j * d + c];
      }
      const int* ri = oi + (long long)q * RowShape::ni;
      r.n_acc[i] = ri[0];
      r.n_rej[i] = ri[1];
      r.n_hits[i] = ri[2];
      r.status[i] = ri[3];
    }
    {
      std::lock_guard<std::mutex> g(mu);
      const auto now = Clock::now();
      for (auto& hq : P.held) {
        Request& r = *hq.first;
        if (++r.done == r.n) {
          r.state = 2;
          r.finished = now;
          latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r.submitted).count());
        }
      }
      P.held.clear();
    }
    cv.notify_all();
  }

  // A pool that failed (lock held): the requests it holds, and those of its
  // problem still waiting, fail.
  void fail_pool(Pool& P, int rc) {
    const auto now = Clock::now();
    auto fail = [&](std::pair<std::shared_ptr<Request>, int>& o) {
      if (!o.first) return;
      Request& r = *o.first;
      if (r.state < 2) {
        r.state = 3;
        r.error = rc;
        r.finished = now;
      }
      o.first.reset();
    };
    for (auto& o : P.owner) fail(o);
    for (auto& o : P.held) fail(o);
    P.held.clear();
    for (auto& r : pending)
      if (same_key(r->key, P.key) && r->state < 2) {
        r->state = 3;
        r->error = rc;
        r->finished = now;
      }
    pending.erase(std::remove_if(pending.begin(), pending.end(),
                                 [](const std::shared_ptr<Request>& r) { return r->state == 3; }),
                  pending.end());
  }

  void run() {
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      // retired pools return their arena blocks and stream
      for (size_t q = 0; q < pools.size();) {
        Pool& P = *pools[q];
        if (P.finished.load()) {
          if (P.runner.joinable()) {
            lk.unlock();
            P.runner.join();
            lk.lock();
          }
          if (P.rc != HG_OK) fail_pool(P, P.rc);
          dev_arena.release(P.dev_off, P.dev_len);
          stg_arena.release(P.stg_off, P.stg_len);
          slot_busy[P.slot] = 0;
          pools.erase(pools.begin() + q);
          cv.notify_all();
        } else {
          ++q;
        }
      }
      if (stop && pending.empty() && pools.empty()) return;
      // open a pool for the oldest waiting problem that has none
      bool opened = false;
      for (auto& r : pending) {
        bool has_pool = false;
        for (auto& P : pools) has_pool |= same_key(P->key, r->key);
        if (has_pool) continue;
        int free_slot = -1;
        for (size_t i = 0; i < slot_busy.size(); ++i)
          if (!slot_busy[i]) {
            free_slot = (int)i;
            break;
          }
        if (free_slot < 0) break;
        const int d = r->key.dim, H = r->key.has_ev ? r->key.ev.max_hits : 0;
        // slots: pool_slots, halved until the free arenas hold the pool
        int C = cfg.pool_slots;
        while (C >= 32) {
          const PoolLayout L(C, d, H);
          if (L.dev_bytes <= dev_arena.largest() && L.stg_bytes <= stg_arena.largest()) break;
          C /= 2;
        }
        if (C < 32) {
          if (pools.empty()) {
            // not even 32 slots fit an idle server: the request cannot run
            auto gone = r;
            gone->state = 3;
            gone->error = HG_ERR_ARGS;
            gone->finished = Clock::now();
            pending.erase(std::find(pending.begin(), pending.end(), gone));
            cv.notify_all();
            opened = true;  // rescan
          }
          break;
        }
        const PoolLayout L(C, d, H);
        std::unique_ptr<Pool> P(new Pool());
        P->key = r->key;
        P->dim = d;
        P->hits = H;
        P->C = C;
        P->slot = free_slot;
        P->dev_len = L.dev_bytes;
        P->stg_len = L.stg_bytes;
        P->dev_off = dev_arena.alloc(L.dev_bytes);
        P->stg_off = P->dev_off >= 0 ? stg_arena.alloc(L.stg_bytes) : -1;
        if (P->dev_off < 0 || P->stg_off < 0) {
          if (P->dev_off >= 0) dev_arena.release(P->dev_off, P->dev_len);
          break;
        }
        P->free_slots.resize(C);
        for (int i = 0; i < C; ++i) P->free_slots[i] = C - 1 - i;  // slot 0 taken first
        P->owner.resize(C);
        slot_busy[free_slot] = 1;
        Pool* pp = P.get();
        pools.push_back(std::move(P));
        pp->runner = std::thread([this, pp] {
          cudaSetDevice(cfg.device);
          pp->rc = run_pool(*pp);
          pp->finished.store(1);
          cv.notify_all();
        });
        opened = true;
        break;  // one at a time: rescan with the new pool in place
      }
      if (!opened) cv.wait_for(lk, std::chrono::microseconds(500));
    }
  }
};

extern "C" {

void hg_serve_config_default(hg_serve_config* c) {
  if (!c) return;
  c->device = 0;
  c->hbm_budget_bytes = 8LL << 30;
  c->max_concurrent = 4;
  c->staging_bytes = 1LL << 30;
  c->pool_slots = 32768;
  c->seg_steps = 16;
}

int hg_serve_create(const hg_serve_config* cfg, hg_server** out) {
  if (!out) return HG_ERR_ARGS;
  *out = nullptr;
  hg_serve_config c;
  hg_serve_config_default(&c);
  if (cfg) c = *cfg;
  if (c.max_concurrent < 1 || c.max_concurrent > 64 || c.hbm_budget_bytes <= 0 || c.staging_bytes <= 0 ||
      c.pool_slots < 32 || c.pool_slots > (1 << 24) || c.seg_steps < 1 || c.seg_steps > (1 << 20))
    return HG_ERR_ARGS;
  std::unique_ptr<hg_server> s(new hg_server());
  s->cfg = c;
  if (cudaSetDevice(c.device) != cudaSuccess) return HG_ERR_NO_DEVICE;
  // a failure part way releases what was made so far (no worker runs yet)
  auto release = [&s](int rc) {
    for (auto st : s->streams) cudaStreamDestroy(st);
    if (s->dev_base) cudaFree(s->dev_base);
    if (s->stg_base) cudaFreeHost(s->stg_base);
    return rc;
  };
  if (cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, c.device) != cudaSuccess || s->sms < 1)
    return release(HG_ERR_NO_DEVICE);
  if (cudaMalloc(&s->dev_base, (size_t)c.hbm_budget_bytes) != cudaSuccess) {
    s->dev_base = nullptr;
    cudaGetLastError();
    return release(HG_ERR_CUDA);
  }
  if (cudaHostAlloc(&s->stg_base, (size_t)c.staging_bytes, cudaHostAllocMapped) != cudaSuccess) {
    s->stg_base = nullptr;
    cudaGetLastError();
    return release(HG_ERR_CUDA);
  }
  // the collection kernel writes finished rows straight into the staging
  if (cudaHostGetDevicePointer((void**)&s->stg_dev, s->stg_base, 0) != cudaSuccess) {
    cudaGetLastError();
    return release(HG_ERR_CUDA);
  }
  s->dev_arena.reset(c.hbm_budget_bytes);
  s->stg_arena.reset(c.staging_bytes);
  for (int i = 0; i < c.max_concurrent; ++i) {
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return release(HG_ERR_CUDA);
    s->streams.push_back(st);
  }
  s->slot_busy.assign(c.max_concurrent, 0);
  hg_server* raw = s.release();
  raw->worker = std::thread([raw] {
    cudaSetDevice(raw->cfg.device);
    raw->run();
  });
  *out = raw;
  return HG_OK;
}

int hg_serve_destroy(hg_server* s) {
  if (!s) return HG_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    s->pending.clear();
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto st : s->streams) cudaStreamDestroy(st);
  if (s->dev_base) cudaFree(s->dev_base);
  if (s->stg_base) cudaFreeHost(s->stg_base);
  delete s;
  return HG_OK;
}

int hg_serve_submit(hg_server* s, double mu, int dim, int N, const double* y0, double t0, double tmax,
                    const hg_dop853_opts* opts, const hg_event* ev, long long* request_id) {
  if (!s || !request_id || !opts || (dim != 6 && dim != 42) || N < 1 || !y0) return HG_ERR_ARGS;
  if (ev && ev->index >= 0 && (ev->index >= dim || ev->max_hits < 1 || ev->direction < -1 || ev->direction > 1))
    return HG_ERR_ARGS;
  if (opts->flip_lo < 0 || opts->flip_hi > dim || opts->flip_lo > opts->flip_hi || !(opts->rtol >= 0.0) ||
      !(opts->atol >= 0.0) || !(opts->min_step > 0.0) || !(opts->max_step > 0.0) || opts->max_steps < 1)
    return HG_ERR_ARGS;
  auto r = std::make_shared<Request>();
  memset(&r->key, 0, sizeof(Key));
  r->key.mu = mu;
  r->key.t0 = t0;
  r->key.tmax = tmax;
  r->key.dim = dim;
  // field by field into the zeroed key: padding bytes stay zero, so equal
  // problems compare equal
  r->key.o.rtol = opts->rtol;
  r->key.o.atol = opts->atol;
  r->key.o.max_step = opts->max_step;
  r->key.o.min_step = opts->min_step;
  r->key.o.max_steps = opts->max_steps;
  r->key.o.fwd = opts->fwd;
  r->key.o.flip_lo = opts->flip_lo;
  r->key.o.flip_hi = opts->flip_hi;
  r->key.has_ev = (ev && ev->index >= 0) ? 1 : 0;
  if (r->key.has_ev) {
    r->key.ev.index = ev->index;
    r->key.ev.offset = ev->offset;
    r->key.ev.direction = ev->direction;
    r->key.ev.max_hits = ev->max_hits;
    r->key.ev.xtol = ev->xtol;
    r->key.ev.gtol = ev->gtol;
  }
  const int H = r->key.has_ev ? r->key.ev.max_hits : 0;
  r->n = N;
  r->y0.assign(y0, y0 + (size_t)N * dim);
  r->y_end.assign((size_t)N * dim, 0.0);
  r->t_end.assign(N, 0.0);
  r->hit_t.assign((size_t)N * H, 0.0);
  r->hit_y.assign((size_t)N * H * dim, 0.0);
  r->n_hits.assign(N, 0);
  r->n_acc.assign(N, 0);
  r->n_rej.assign(N, 0);
  r->status.assign(N, 0);
  r->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) return HG_ERR_ARGS;
    r->id = s->next_id++;
    s->all[r->id] = r;
    s->pending.push_back(r);
    *request_id = r->id;
  }
  s->cv.notify_all();
  return HG_OK;
}

int hg_serve_poll(hg_server* s, long long id, int* state) {
  if (!s || !state) return HG_ERR_ARGS;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return HG_ERR_ARGS;
  *state = it->second->state;
  return HG_OK;
}

int hg_serve_wait(hg_server* s, long long id, double timeout_s) {
  if (!s) return HG_ERR_ARGS;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return HG_ERR_ARGS;
  auto r = it->second;
  const auto until = Clock::now() + std::chrono::duration<double>(timeout_s);
  while (r->state < 2) {
    if (s->cv.wait_until(lk, until) == std::cv_status::timeout && r->state < 2) return HG_ERR_TIMEOUT;
  }
  return r->state == 2 ? HG_OK : r->error;
}

int hg_serve_fetch(hg_server* s, long long id, double* y_end, double* t_end, double* hit_t, double* hit_y,
                   int* n_hits, int* n_accept, int* n_reject, int* status) {
  if (!s) return HG_ERR_ARGS;
  std::shared_ptr<Request> r;
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end() || it->second->state < 2) return HG_ERR_ARGS;
    r = it->second;
    s->all.erase(it);
  }
  if (r->state == 3) return r->error;
  const int n = r->n, d = r->key.dim;
  const size_t hits = r->key.has_ev ? (size_t)r->key.ev.max_hits : 0;
  if (y_end) memcpy(y_end, r->y_end.data(), 8ull * n * d);
  if (t_end) memcpy(t_end, r->t_end.data(), 8ull * n);
  if (hit_t && hits) memcpy(hit_t, r->hit_t.data(), 8ull * n * hits);
  if (hit_y && hits) memcpy(hit_y, r->hit_y.data(), 8ull * n * hits * d);
  if (n_hits) memcpy(n_hits, r->n_hits.data(), 4ull * n);
  if (n_accept) memcpy(n_accept, r->n_acc.data(), 4ull * n);
  if (n_reject) memcpy(n_reject, r->n_rej.data(), 4ull * n);
  if (status) memcpy(status, r->status.data(), 4ull * n);
  return HG_OK;
}

int hg_serve_cancel(hg_server* s, long long id) {
  if (!s) return HG_ERR_ARGS;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end() || it->second->state != 0) return HG_ERR_ARGS;
  auto r = it->second;
  s->pending.erase(std::remove(s->pending.begin(), s->pending.end(), r), s->pending.end());
  s->all.erase(it);
  return HG_OK;
}

int hg_serve_stats(hg_server* s, double* p50_ms, double* p99_ms, long long* requests, long long* batches) {
  if (!s) return HG_ERR_ARGS;
  std::vector<double> v;
  {
    std::lock_guard<std::mutex> g(s->mu);
    v = s->latencies_ms;
    if (batches) *batches = s->segments;
  }
  if (requests) *requests = (long long)v.size();
  auto pct = [&](double q) {
    if (v.empty()) return 0.0;
    std::vector<double> w = v;
    const size_t k = std::min(w.size() - 1, (size_t)(q * (double)(w.size() - 1) + 0.5));
    std::nth_element(w.begin(), w.begin() + k, w.end());
    return w[k];
  };
  if (p50_ms) *p50_ms = pct(0.50);
  if (p99_ms) *p99_ms = pct(0.99);
  return HG_OK;
}

}  // extern "C"
