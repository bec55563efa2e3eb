// Native request server for DOP853 propagation requests (continuous
// batching).  Requests are host arrays; a worker thread merges every pending
// request that shares a problem (mu, dim, span, options, event) into one
// batch, admits batches while their device footprint fits the device arena,
// runs them concurrently on its own streams and handles (host-scheduled
// segments for wide 6-dim batches, one segment that finishes every
// trajectory otherwise), and parks each request's results on the host until
// it is fetched.  Results are those of a direct hg_propagate_dop853 call on
// the request alone: trajectories never interact.
//
// Memory: hg_serve_create allocates a device arena of hbm_budget_bytes and a
// pinned host staging arena of staging_bytes; every batch takes one block of
// each (its inputs, outputs and segment workspace on the device; its inputs
// and outputs in pinned memory, so its copies run asynchronously on its
// stream) and returns them when it finishes, on success or failure.  Nothing
// is allocated after creation.
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

#include "hitengpu.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Key {
  double mu, t0, tmax;
  int dim;
  hg_dop853_opts o;
  int has_ev;
  hg_event ev;
  bool operator<(const Key& b) const { return memcmp(this, &b, sizeof(Key)) < 0; }
};

struct Request {
  long long id;
  Key key;
  int n;
  std::vector<double> y0;  // row-major (n, dim)
  // results
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
    size_ = size;
    free_.clear();
    if (size > 0) free_[0] = size;
  }
  long long size() const { return size_; }
  // offset of a block of `bytes` (256-byte aligned), or -1
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
  static long long up(long long x) { return (x + 255) & ~255LL; }
  long long free_bytes() const {
    long long t = 0;
    for (const auto& f : free_) t += f.second;
    return t;
  }

 private:
  long long size_ = 0;
  std::map<long long, long long> free_;  // offset -> length, disjoint, not adjacent
};

// Layout of a batch of n trajectories: the inputs and outputs (the same
// layout on the device and in pinned staging) and, on the device only, the
// segment workspace.  y0 [d][n]; outputs y_end [d][n], t_end [n],
// hit_t [hits][n], hit_y [hits][d][n], then four int arrays [n].
struct Layout {
  long long off_ye, off_te, off_ht, off_hy, off_i, io_bytes, ws_bytes;
  Layout(int d, int n, int hits) {
    const long long nn = n;
    off_ye = Arena::up(8 * d * nn);
    off_te = off_ye + 8 * d * nn;
    off_ht = off_te + 8 * nn;
    off_hy = off_ht + 8 * hits * nn;
    off_i = off_hy + 8 * (long long)hits * d * nn;
    io_bytes = Arena::up(off_i + 16 * nn);
    ws_bytes = Arena::up(hg_dop853_segmented_workspace_bytes(n, d, hits));
  }
  long long device_bytes() const { return io_bytes + ws_bytes; }
  long long out_bytes() const { return io_bytes - off_ye; }
};

struct Batch {
  Key key;
  std::vector<std::shared_ptr<Request>> reqs;
  int n = 0;
  int slot = -1;
  long long dev_off = -1, dev_len = 0, stg_off = -1, stg_len = 0;  // arena blocks
  std::atomic<int> finished{0};
  std::thread runner;
  int rc = HG_OK;
};

}  // namespace

struct hg_server {
  hg_serve_config cfg;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<Request>> pending;
  std::map<long long, std::shared_ptr<Request>> all;
  std::vector<std::unique_ptr<Batch>> running;
  std::vector<cudaStream_t> streams;
  std::vector<hg_handle*> handles;
  std::vector<char> slot_busy;
  long long next_id = 1;
  char* dev_base = nullptr;  // device arena (hbm_budget_bytes)
  char* stg_base = nullptr;  // pinned staging arena (staging_bytes)
  Arena dev_arena, stg_arena;
  bool stop = false;
  std::thread worker;
  std::vector<double> latencies_ms;
  long long batches = 0;

  // Copies in, propagation and copies out of one admitted batch on its
  // slot's stream (runs on the batch's own thread; the blocks are owned by
  // the batch and returned in finish()).
  int launch(Batch& b) {
    const Key& k = b.key;
    const int d = k.dim, n = b.n;
    const int hits = k.has_ev ? k.ev.max_hits : 0;
    const Layout L(d, n, hits);
    cudaStream_t s = streams[b.slot];
    if (cudaSetDevice(cfg.device) != cudaSuccess) return HG_ERR_CUDA;
    char* dev = dev_base + b.dev_off;
    char* stg = stg_base + b.stg_off;
    double* h_y0 = (double*)stg;
    int o = 0;
    for (auto& r : b.reqs) {
      for (int i = 0; i < r->n; ++i)
        for (int c = 0; c < d; ++c) h_y0[(size_t)c * n + o + i] = r->y0[(size_t)i * d + c];
      o += r->n;
    }
    if (cudaMemcpyAsync(dev, stg, 8ull * d * n, cudaMemcpyHostToDevice, s) != cudaSuccess) return HG_ERR_CUDA;
    double* ye = (double*)(dev + L.off_ye);
    double* te = (double*)(dev + L.off_te);
    double* ht = hits ? (double*)(dev + L.off_ht) : nullptr;
    double* hy = hits ? (double*)(dev + L.off_hy) : nullptr;
    int* nh = (int*)(dev + L.off_i);
    int* na = nh + n;
    int* nr = na + n;
    int* st = nr + n;
    void* ws = dev + L.io_bytes;
    if (hits && cudaMemsetAsync(ht, 0xFF, 8ull * hits * n * (1 + d), s) != cudaSuccess) return HG_ERR_CUDA;
    if (!hits && cudaMemsetAsync(nh, 0, 4ull * n, s) != cudaSuccess) return HG_ERR_CUDA;
    int rc;
    if (d == 6 && n >= 4096) {
      // wide batches: host-scheduled segments (synchronous on this stream)
      rc = hg_propagate_dop853_scheduled(handles[b.slot], k.mu, d, n, (const double*)dev, n, nullptr, nullptr, k.t0,
                                         k.tmax, &k.o, k.has_ev ? &k.ev : nullptr, 0, 0, nullptr, ye, te, ht, hy,
                                         hits ? nh : nullptr, na, nr, st, ws, L.ws_bytes, s);
    } else {
      // one segment long enough to finish every trajectory (same results as
      // a single pass; the event records live in the batch's workspace)
      const long long seg = std::min<long long>(k.o.max_steps + 1, INT_MAX);
      rc = hg_propagate_dop853_segmented(handles[b.slot], k.mu, d, n, (const double*)dev, n, nullptr, nullptr, k.t0,
                                         k.tmax, &k.o, k.has_ev ? &k.ev : nullptr, 0, 0, nullptr, ye, te, ht, hy,
                                         hits ? nh : nullptr, na, nr, st, (int)seg, 1, 0, ws, L.ws_bytes, s);
    }
    if (rc != HG_OK) {
      cudaStreamSynchronize(s);
      return rc;
    }
    if (cudaMemcpyAsync(stg + L.off_ye, dev + L.off_ye, (size_t)L.out_bytes(), cudaMemcpyDeviceToHost, s) !=
        cudaSuccess) {
      cudaStreamSynchronize(s);
      return HG_ERR_CUDA;
    }
    return cudaStreamSynchronize(s) == cudaSuccess ? HG_OK : HG_ERR_CUDA;
  }

  // scatter a finished batch to its requests (called with the lock held)
  void finish(Batch& b) {
    const int d = b.key.dim, n = b.n, hits = b.key.has_ev ? b.key.ev.max_hits : 0;
    const Layout L(d, n, hits);
    const char* stg = stg_base + b.stg_off;
    const double* h_yend = (const double*)(stg + L.off_ye);
    const double* h_tend = (const double*)(stg + L.off_te);
    const double* h_hitt = (const double*)(stg + L.off_ht);
    const double* h_hity = (const double*)(stg + L.off_hy);
    const int* h_nh = (const int*)(stg + L.off_i);
    const int* h_na = h_nh + n;
    const int* h_nr = h_na + n;
    const int* h_st = h_nr + n;
    const auto now = Clock::now();
    int o = 0;
    for (auto& r : b.reqs) {
      const int m = r->n;
      if (b.rc == HG_OK) {
        r->y_end.resize((size_t)m * d);
        r->t_end.resize(m);
        r->n_hits.resize(m);
        r->n_acc.resize(m);
        r->n_rej.resize(m);
        r->status.resize(m);
        r->hit_t.resize((size_t)m * hits);
        r->hit_y.resize((size_t)m * hits * d);
        for (int i = 0; i < m; ++i) {
          const int g = o + i;
          for (int c = 0; c < d; ++c) r->y_end[(size_t)i * d + c] = h_yend[(size_t)c * n + g];
          r->t_end[i] = h_tend[g];
          r->n_hits[i] = hits ? h_nh[g] : 0;
          r->n_acc[i] = h_na[g];
          r->n_rej[i] = h_nr[g];
          r->status[i] = h_st[g];
          for (int j = 0; j < hits; ++j) {
            r->hit_t[(size_t)i * hits + j] = h_hitt[(size_t)j * n + g];
            for (int c = 0; c < d; ++c)
              r->hit_y[((size_t)i * hits + j) * d + c] = h_hity[((size_t)j * d + c) * n + g];
          }
        }
        r->state = 2;
      } else {
        r->state = 3;
        r->error = b.rc;
      }
      r->finished = now;
      latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r->submitted).count());
      o += m;
    }
    dev_arena.release(b.dev_off, b.dev_len);
    stg_arena.release(b.stg_off, b.stg_len);
    slot_busy[b.slot] = 0;
    ++batches;
  }

  // A request that can never fit the arenas fails at once (lock held).
  void reject(const std::shared_ptr<Request>& r) {
    r->state = 3;
    r->error = HG_ERR_ARGS;
    r->finished = Clock::now();
    latencies_ms.push_back(std::chrono::duration<double, std::milli>(r->finished - r->submitted).count());
  }

  long long dev_free_bytes() const { return free_total(dev_arena); }
  long long stg_free_bytes() const { return free_total(stg_arena); }
  static long long free_total(const Arena& a) { return a.free_bytes(); }

  void run() {
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      // completed batches
      for (size_t q = 0; q < running.size();) {
        Batch& b = *running[q];
        if (b.finished.load()) {
          if (b.runner.joinable()) b.runner.join();
          finish(b);
          running.erase(running.begin() + q);
          cv.notify_all();
        } else {
          ++q;
        }
      }
      if (stop && pending.empty() && running.empty()) return;
      // admit: merge pending requests per problem, in arrival order, while
      // the merged batches' blocks fit what the arenas have free
      std::vector<std::unique_ptr<Batch>> admit;
      if (!pending.empty()) {
        std::map<Key, Batch*> open;
        std::deque<std::shared_ptr<Request>> keep;
        long long dev_free = dev_free_bytes(), stg_free = stg_free_bytes();
        for (auto& r : pending) {
          const int hits = r->key.has_ev ? r->key.ev.max_hits : 0;
          const Layout alone(r->key.dim, r->n, hits);
          if (alone.device_bytes() > dev_arena.size() || alone.io_bytes > stg_arena.size()) {
            reject(r);
            continue;
          }
          auto it = open.find(r->key);
          Batch* b = it == open.end() ? nullptr : it->second;
          const Layout before(r->key.dim, b ? b->n : 0, hits), after(r->key.dim, (b ? b->n : 0) + r->n, hits);
          const long long dd = b ? after.device_bytes() - before.device_bytes() : after.device_bytes();
          const long long ds = b ? after.io_bytes - before.io_bytes : after.io_bytes;
          int free_slot = -1;
          if (!b) {
            for (size_t sidx = 0; sidx < slot_busy.size(); ++sidx)
              if (!slot_busy[sidx]) {
                bool taken = false;
                for (auto& a : admit) taken |= a->slot == (int)sidx;
                if (!taken) {
                  free_slot = (int)sidx;
                  break;
                }
              }
          }
          if (dd <= dev_free && ds <= stg_free && (b || free_slot >= 0)) {
            if (!b) {
              admit.emplace_back(new Batch());
              b = admit.back().get();
              b->key = r->key;
              b->slot = free_slot;
              open[r->key] = b;
            }
            b->reqs.push_back(r);
            b->n += r->n;
            dev_free -= dd;
            stg_free -= ds;
          } else {
            keep.push_back(r);
          }
        }
        // blocks for the admitted batches; a batch that does not fit the free
        // blocks (fragmentation) goes back to waiting, in arrival order
        std::vector<std::unique_ptr<Batch>> placed;
        std::deque<std::shared_ptr<Request>> back;
        for (auto& b : admit) {
          const int hits = b->key.has_ev ? b->key.ev.max_hits : 0;
          const Layout L(b->key.dim, b->n, hits);
          b->dev_len = L.device_bytes();
          b->stg_len = L.io_bytes;
          b->dev_off = dev_arena.alloc(b->dev_len);
          b->stg_off = b->dev_off >= 0 ? stg_arena.alloc(b->stg_len) : -1;
          if (b->dev_off < 0 || b->stg_off < 0) {
            if (b->dev_off >= 0) dev_arena.release(b->dev_off, b->dev_len);
            for (auto& r : b->reqs) back.push_back(r);
            continue;
          }
          for (auto& r : b->reqs) r->state = 1;
          placed.push_back(std::move(b));
        }
        if (!back.empty()) {
          // restore arrival order among the requests sent back and those kept
          for (auto& r : keep) back.push_back(r);
          std::stable_sort(back.begin(), back.end(),
                           [](const std::shared_ptr<Request>& x, const std::shared_ptr<Request>& y) {
                             return x->id < y->id;
                           });
          keep.swap(back);
        }
        pending.swap(keep);
        admit.swap(placed);
      }
      for (auto& b : admit) {
        slot_busy[b->slot] = 1;
        Batch* bp = b.get();
        // each batch runs on its own thread (the scheduled driver waits on
        // its stream); completion wakes this loop
        bp->runner = std::thread([this, bp] {
          cudaSetDevice(cfg.device);
          bp->rc = launch(*bp);
          bp->finished.store(1);
          cv.notify_all();
        });
        running.push_back(std::move(b));
      }
      if (admit.empty()) cv.wait_for(lk, std::chrono::microseconds(500));
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
}

int hg_serve_create(const hg_serve_config* cfg, hg_server** out) {
  if (!out) return HG_ERR_ARGS;
  *out = nullptr;
  hg_serve_config c;
  hg_serve_config_default(&c);
  if (cfg) c = *cfg;
  if (c.max_concurrent < 1 || c.max_concurrent > 64 || c.hbm_budget_bytes <= 0 || c.staging_bytes <= 0)
    return HG_ERR_ARGS;
  std::unique_ptr<hg_server> s(new hg_server());
  s->cfg = c;
  if (cudaSetDevice(c.device) != cudaSuccess) return HG_ERR_NO_DEVICE;
  // a failure part way releases what was made so far (no worker runs yet)
  auto release = [&s](int rc) {
    for (auto h : s->handles) hg_destroy(h);
    for (auto st : s->streams) cudaStreamDestroy(st);
    if (s->dev_base) cudaFree(s->dev_base);
    if (s->stg_base) cudaFreeHost(s->stg_base);
    return rc;
  };
  if (cudaMalloc(&s->dev_base, (size_t)c.hbm_budget_bytes) != cudaSuccess) {
    s->dev_base = nullptr;
    cudaGetLastError();
    return release(HG_ERR_CUDA);
  }
  if (cudaHostAlloc(&s->stg_base, (size_t)c.staging_bytes, cudaHostAllocDefault) != cudaSuccess) {
    s->stg_base = nullptr;
    cudaGetLastError();
    return release(HG_ERR_CUDA);
  }
  s->dev_arena.reset(c.hbm_budget_bytes);
  s->stg_arena.reset(c.staging_bytes);
  for (int i = 0; i < c.max_concurrent; ++i) {
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return release(HG_ERR_CUDA);
    s->streams.push_back(st);
    hg_handle* h = nullptr;
    hg_config hc{c.device};
    const int rc = hg_create(&hc, &h);
    if (rc != HG_OK) return release(rc);
    s->handles.push_back(h);
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
  for (auto h : s->handles) hg_destroy(h);
  for (auto st : s->streams) cudaStreamDestroy(st);
  if (s->dev_base) cudaFree(s->dev_base);
  if (s->stg_base) cudaFreeHost(s->stg_base);
  delete s;
  return HG_OK;
}

int hg_serve_submit(hg_server* s, double mu, int dim, int N, const double* y0, double t0, double tmax,
                    const hg_dop853_opts* opts, const hg_event* ev, long long* request_id) {
  if (!s || !request_id || !opts || (dim != 6 && dim != 42) || N < 1 || !y0) return HG_ERR_ARGS;
  if (ev && ev->index >= 0 && (ev->index >= dim || ev->max_hits < 1)) return HG_ERR_ARGS;
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
  r->n = N;
  r->y0.assign(y0, y0 + (size_t)N * dim);
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
    if (batches) *batches = s->batches;
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
