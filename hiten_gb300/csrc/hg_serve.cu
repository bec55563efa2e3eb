// Native request server for DOP853 propagation requests (continuous
// batching).  Requests are host arrays; a worker thread merges every pending
// request that shares a problem (mu, dim, span, options, event) into one
// batch, admits batches while their device footprint fits the budget, runs
// them concurrently on its own streams and handles (host-scheduled segments
// for wide 6-dim batches), and parks each request's results on the host
// until it is fetched.  Results are those of a direct hg_propagate_dop853
// call on the request alone: trajectories never interact.
#include <cuda_runtime.h>
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

struct Batch {
  Key key;
  std::vector<std::shared_ptr<Request>> reqs;
  int n = 0;
  long long bytes = 0;
  int slot = -1;
  void* dev = nullptr;
  std::vector<double> h_y0, h_yend, h_tend, h_hitt, h_hity;
  std::vector<int> h_nh, h_na, h_nr, h_st;
  std::atomic<int> finished{0};
  std::thread runner;
  int rc = HG_OK;
};

long long batch_bytes(int dim, int n, int hits) {
  const long long per = 8LL * dim * 2 + 8 + 4 * 4 + (hits > 0 ? (8LL + 8LL * dim) * hits : 0);
  return per * n + (hits > 0 ? (15LL * dim + 3) * 8 * (long long)n * hits : 0) + 4096;
}

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
  long long in_use = 0;
  bool stop = false;
  std::thread worker;
  std::vector<double> latencies_ms;
  long long batches = 0;

  int launch(Batch& b) {
    const Key& k = b.key;
    const int d = k.dim, n = b.n;
    const int hits = k.has_ev ? k.ev.max_hits : 0;
    // device layout: y0, y_end [d][n]; t_end [n]; hit_t [hits][n]; hit_y [hits][d][n]; 4 int arrays [n]
    const size_t off_y0 = 0, off_ye = off_y0 + 8ull * d * n, off_te = off_ye + 8ull * d * n,
                 off_ht = off_te + 8ull * n, off_hy = off_ht + 8ull * hits * n, off_i = off_hy + 8ull * hits * d * n;
    const size_t total = off_i + 16ull * n + 256;
    cudaStream_t s = streams[b.slot];
    cudaSetDevice(cfg.device);
    if (cudaMallocAsync(&b.dev, total, s) != cudaSuccess) return HG_ERR_CUDA;
    char* base = (char*)b.dev;
    b.h_y0.assign((size_t)d * n, 0.0);
    int o = 0;
    for (auto& r : b.reqs) {
      for (int i = 0; i < r->n; ++i)
        for (int c = 0; c < d; ++c) b.h_y0[(size_t)c * n + o + i] = r->y0[(size_t)i * d + c];
      o += r->n;
    }
    if (cudaMemcpyAsync(base + off_y0, b.h_y0.data(), 8ull * d * n, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return HG_ERR_CUDA;
    double* ye = (double*)(base + off_ye);
    double* te = (double*)(base + off_te);
    double* ht = hits ? (double*)(base + off_ht) : nullptr;
    double* hy = hits ? (double*)(base + off_hy) : nullptr;
    int* nh = (int*)(base + off_i);
    int* na = nh + n;
    int* nr = na + n;
    int* st = nr + n;
    if (hits && cudaMemsetAsync(ht, 0xFF, 8ull * hits * n * (1 + d), s) != cudaSuccess) return HG_ERR_CUDA;
    int rc = HG_OK;
    if (d == 6 && n >= 4096) {
      // wide batches: host-scheduled segments (synchronous on this stream)
      const long long wsb = hg_dop853_segmented_workspace_bytes(n, d, hits);
      void* ws = nullptr;
      if (cudaMallocAsync(&ws, (size_t)wsb, s) != cudaSuccess) return HG_ERR_CUDA;
      rc = hg_propagate_dop853_scheduled(handles[b.slot], k.mu, d, n, (const double*)(base + off_y0), n, nullptr,
                                         nullptr, k.t0, k.tmax, &k.o, k.has_ev ? &k.ev : nullptr, 0, 0, nullptr, ye,
                                         te, ht, hy, nh, na, nr, st, ws, wsb, s);
      cudaFreeAsync(ws, s);
    } else {
      rc = hg_propagate_dop853(handles[b.slot], k.mu, d, n, (const double*)(base + off_y0), n, nullptr, nullptr,
                               k.t0, k.tmax, &k.o, k.has_ev ? &k.ev : nullptr, 0, 0, nullptr, ye, te, ht, hy, nh, na,
                               nr, st, s);
    }
    if (rc != HG_OK) {
      cudaFreeAsync(b.dev, s);
      b.dev = nullptr;
      cudaStreamSynchronize(s);
      return rc;
    }
    b.h_yend.resize((size_t)d * n);
    b.h_tend.resize(n);
    b.h_hitt.resize((size_t)hits * n);
    b.h_hity.resize((size_t)hits * d * n);
    b.h_nh.resize(n);
    b.h_na.resize(n);
    b.h_nr.resize(n);
    b.h_st.resize(n);
    if (cudaMemcpyAsync(b.h_yend.data(), ye, 8ull * d * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(b.h_tend.data(), te, 8ull * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(b.h_nh.data(), nh, 4ull * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(b.h_na.data(), na, 4ull * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(b.h_nr.data(), nr, 4ull * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(b.h_st.data(), st, 4ull * n, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return HG_ERR_CUDA;
    if (hits && (cudaMemcpyAsync(b.h_hitt.data(), ht, 8ull * hits * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                 cudaMemcpyAsync(b.h_hity.data(), hy, 8ull * hits * d * n, cudaMemcpyDeviceToHost, s) !=
                     cudaSuccess))
      return HG_ERR_CUDA;
    cudaFreeAsync(b.dev, s);
    b.dev = nullptr;
    return cudaStreamSynchronize(s) == cudaSuccess ? HG_OK : HG_ERR_CUDA;
  }

  // scatter a finished batch to its requests (called with the lock held)
  void finish(Batch& b) {
    const int d = b.key.dim, n = b.n, hits = b.key.has_ev ? b.key.ev.max_hits : 0;
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
          for (int c = 0; c < d; ++c) r->y_end[(size_t)i * d + c] = b.h_yend[(size_t)c * n + g];
          r->t_end[i] = b.h_tend[g];
          r->n_hits[i] = hits ? b.h_nh[g] : 0;
          r->n_acc[i] = b.h_na[g];
          r->n_rej[i] = b.h_nr[g];
          r->status[i] = b.h_st[g];
          for (int j = 0; j < hits; ++j) {
            r->hit_t[(size_t)i * hits + j] = b.h_hitt[(size_t)j * n + g];
            for (int c = 0; c < d; ++c)
              r->hit_y[((size_t)i * hits + j) * d + c] = b.h_hity[((size_t)j * d + c) * n + g];
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
    in_use -= b.bytes;
    slot_busy[b.slot] = 0;
    ++batches;
  }

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
      // admit: merge pending requests per problem, in arrival order
      std::vector<std::unique_ptr<Batch>> admit;
      if (!pending.empty()) {
        std::map<Key, Batch*> open;
        std::deque<std::shared_ptr<Request>> keep;
        long long budget = cfg.hbm_budget_bytes - in_use;
        for (auto& r : pending) {
          const int hits = r->key.has_ev ? r->key.ev.max_hits : 0;
          const long long bytes = batch_bytes(r->key.dim, r->n, hits);
          auto it = open.find(r->key);
          Batch* b = it == open.end() ? nullptr : it->second;
          const bool room = bytes <= budget || (in_use == 0 && admit.empty() && b == nullptr);
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
          if (room && (b || free_slot >= 0)) {
            if (!b) {
              admit.emplace_back(new Batch());
              b = admit.back().get();
              b->key = r->key;
              b->slot = free_slot;
              open[r->key] = b;
            }
            b->reqs.push_back(r);
            b->n += r->n;
            b->bytes += bytes;
            budget -= bytes;
            r->state = 1;
          } else {
            keep.push_back(r);
          }
        }
        pending.swap(keep);
      }
      for (auto& b : admit) {
        slot_busy[b->slot] = 1;
        in_use += b->bytes;
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
}

int hg_serve_create(const hg_serve_config* cfg, hg_server** out) {
  if (!out) return HG_ERR_ARGS;
  *out = nullptr;
  hg_serve_config c;
  hg_serve_config_default(&c);
  if (cfg) c = *cfg;
  if (c.max_concurrent < 1 || c.max_concurrent > 64 || c.hbm_budget_bytes <= 0) return HG_ERR_ARGS;
  std::unique_ptr<hg_server> s(new hg_server());
  s->cfg = c;
  if (cudaSetDevice(c.device) != cudaSuccess) return HG_ERR_NO_DEVICE;
  // a failure part way releases the streams and handles made so far (no worker runs yet)
  auto release = [&s](int rc) {
    for (auto h : s->handles) hg_destroy(h);
    for (auto st : s->streams) cudaStreamDestroy(st);
    return rc;
  };
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
