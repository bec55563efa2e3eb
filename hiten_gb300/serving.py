"""Continuous-batching request server for manifold, correction and
section-map solves (FP64, one GPU).

Requests arrive at any time.  Every scheduler tick the engine:

1. admits waiting requests in arrival order while their HBM footprint fits
   the budget (a request that does not fit waits until running batches
   release memory);
2. merges the admitted requests of one kind into one batch and launches it
   on its own CUDA stream, so batches of different kinds, and batches admitted
   while others are still running, execute concurrently on the device;
3. collects finished batches, splits the results back per request, releases
   their memory and stamps the completion time.

With ``slots=True`` the propagating kinds (manifold, synodic) go instead to
the library's native request server (``NativeServer`` over ``hg_serve_*``):
each problem runs in a pool of device-resident trajectory slots, and the
trajectories of a request that arrives while others run enter the pool at
the next segment boundary as slots free up (lane-level admission; one host
synchronisation per segment).  Corrections keep the merged batches.

Trajectories are independent lanes in every kernel, so a request's result
does not depend on what it was batched with (checked bit for bit by
tests/test_gpu_serving.py in both forms).  `run_sequential` is the plain
form: one request at a time, each with its own kernel calls, on one stream.

Request kinds (types/services: manifold.py:293-442, orbits.py:114-151;
poincare/synodic): 'manifold' (seeds, DOP853 1e-12 backward to t = -8 or the
x = 1 - mu plane), 'correct' (halo guesses, batched Newton), 'synodic'
(states, DOP853 1e-11 to t = 20, up to 8 decreasing y = 0 crossings).
"""
import concurrent.futures as cf
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import corrector
from . import propagate as P

BYTES_PER_TRAJ = {"manifold": 8 * (6 + 6 + 1 + 7) + 4 * 4,
                  "synodic": 8 * (6 + 6 + 1 + 8 * 7) + 4 * 4,
                  "correct": 8 * (42 * 3 + 6 * 4) + 4 * 4}


@dataclass
class Request:
    rid: int
    kind: str
    payload: np.ndarray
    arrival: float = 0.0
    admitted: float = None
    done: float = None
    result: dict = None

    @property
    def footprint(self):
        return BYTES_PER_TRAJ[self.kind] * len(self.payload)


def _solve(kind, x, mu, device, batched=True):
    """Run one batch of one kind; returns host arrays per trajectory.
    `batched` = False is the plain form: one single-pass call, no scheduling."""
    sched = batched and len(x) >= P.SCHEDULE_MIN
    if kind == "manifold":
        ev = P.EventSpec(index=0, offset=1.0 - mu, direction=0, max_hits=1)
        r = P.propagate_dop853(x, 0.0, 8.0, mu, rtol=1e-12, atol=1e-12, max_step=1e4, fwd=-1, flip=(0, 6),
                               event=ev, device=device, scheduled=sched)
        return {"y_end": r.y_end.cpu().numpy(), "t_end": r.t_end.cpu().numpy(), "n_hits": r.n_hits.cpu().numpy(),
                "hit_t": r.hit_t.cpu().numpy(), "hit_y": r.hit_y.cpu().numpy(), "n_accept": r.n_accept.cpu().numpy(),
                "status": r.status.cpu().numpy()}
    if kind == "synodic":
        ev = P.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
        r = P.propagate_dop853(x, 0.0, 20.0, mu, rtol=1e-11, atol=1e-11, max_step=1e4, event=ev, device=device,
                               scheduled=sched)
        return {"y_end": r.y_end.cpu().numpy(), "n_hits": r.n_hits.cpu().numpy(), "hit_t": r.hit_t.cpu().numpy(),
                "hit_y": r.hit_y.cpu().numpy(), "n_accept": r.n_accept.cpu().numpy(), "status": r.status.cpu().numpy()}
    if kind == "correct":
        res = corrector.correct_halo(x, mu, device=device)
        return {"x0": res.x0, "period": res.period, "iterations": res.iterations, "status": res.status}
    raise ValueError(kind)


# The propagation problem of each propagating request kind: (t span, keyword
# arguments of propagate_dop853 / NativeServer.submit), as _solve runs it.
def _problem(kind, mu):
    if kind == "manifold":
        return 8.0, dict(rtol=1e-12, atol=1e-12, max_step=1e4, fwd=-1, flip=(0, 6),
                         event=P.EventSpec(index=0, offset=1.0 - mu, direction=0, max_hits=1))
    return 20.0, dict(rtol=1e-11, atol=1e-11, max_step=1e4, event=P.EventSpec(index=1, offset=0.0, direction=-1,
                                                                                max_hits=8))


def _native_result(kind, f):
    """A request's rows from the native server in _solve's form (crossing
    entries past each trajectory's count are NaN, as the direct call leaves them)."""
    ht, hy = f["hit_t"].copy(), f["hit_y"].copy()
    unused = np.arange(ht.shape[1])[None, :] >= f["n_hits"][:, None]
    ht[unused] = np.nan
    hy[unused] = np.nan
    out = {"y_end": f["y_end"], "n_hits": f["n_hits"], "hit_t": ht, "hit_y": hy, "n_accept": f["n_accept"],
           "status": f["status"]}
    if kind == "manifold":
        out = {"y_end": f["y_end"], "t_end": f["t_end"], "n_hits": f["n_hits"], "hit_t": ht, "hit_y": hy,
               "n_accept": f["n_accept"], "status": f["status"]}
    return out


def _split(kind, res, sizes):
    out, off = [], 0
    for n in sizes:
        out.append({k: v[off:off + n] for k, v in res.items()})
        off += n
    return out


def admit(waiting, in_use, budget, free_streams):
    """One admission pass over `waiting` (in arrival order): a request joins
    the batch of its kind while its footprint fits the budget (the first one
    always fits an idle device, so an oversized request cannot starve), and a
    new kind opens a batch only while a stream is free for it.  Returns
    ({kind: [requests]}, still waiting, bytes in use); admitted requests get
    their admission time."""
    admitted = {}
    keep = []
    for r in waiting:
        fits = in_use + r.footprint <= budget or (in_use == 0 and not admitted)
        if fits and (r.kind in admitted or len(admitted) < free_streams):
            admitted.setdefault(r.kind, []).append(r)
            in_use += r.footprint
            r.admitted = time.perf_counter()
        else:
            keep.append(r)
    return admitted, keep, in_use


@dataclass
class ServingStats:
    n: int = 0
    wall_s: float = 0.0
    latencies: list = field(default_factory=list)
    traj_steps: int = 0
    batches: int = 0

    def summary(self):
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return {"requests": self.n, "wall_s": self.wall_s, "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "traj_steps": self.traj_steps,
                "traj_steps_per_s": self.traj_steps / self.wall_s if self.wall_s else 0.0,
                "requests_per_s": self.n / self.wall_s if self.wall_s else 0.0, "batches": self.batches}


class ServingEngine:
    """Continuous batching with HBM-footprint admission (see module docstring).

    ``slots=True``: manifold and synodic requests go to the library's native
    server (``NativeServer``), where each kind runs in a pool of
    device-resident trajectory slots that arriving requests enter at every
    segment boundary as slots free up (lane-level admission; the budget is
    the server's device arena); correction requests keep the per-tick merged
    batches."""

    def __init__(self, mu, device=None, hbm_budget_bytes=8 << 30, max_concurrent=6, tick_s=0.002, slots=False,
                 pool_slots=32768, seg_steps=16):
        self.mu = float(mu)
        self.device = P._device(device)
        self.budget = int(hbm_budget_bytes)
        self.in_use = 0
        self.tick_s = tick_s
        self.pool = cf.ThreadPoolExecutor(max_workers=max_concurrent)
        self.max_concurrent = max_concurrent
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(max_concurrent)]
        self.free_streams = list(range(max_concurrent))
        self.lock = threading.Lock()
        self.native = None
        if slots:
            self.native = NativeServer(device=self.device.index or 0, hbm_budget_bytes=self.budget,
                                       max_concurrent=2, pool_slots=pool_slots, seg_steps=seg_steps)

    def _run_batch(self, kind, reqs, sidx):
        x = np.concatenate([r.payload for r in reqs])
        with torch.cuda.stream(self.streams[sidx]):
            res = _solve(kind, x, self.mu, self.device)
            torch.cuda.current_stream(self.device).synchronize()
        t = time.perf_counter()
        for r, part in zip(reqs, _split(kind, res, [len(q.payload) for q in reqs])):
            r.result = part
            r.done = t
        return kind, reqs, sidx

    def serve(self, requests, t0=None):
        """Serve `requests` (sorted by `arrival`, seconds relative to t0)."""
        t0 = time.perf_counter() if t0 is None else t0
        waiting = []
        futures = set()
        in_server = {}  # native request id -> request
        nxt = 0
        stats = ServingStats()
        while nxt < len(requests) or waiting or futures or in_server:
            now = time.perf_counter() - t0
            while nxt < len(requests) and requests[nxt].arrival <= now:
                r = requests[nxt]
                nxt += 1
                if self.native is not None and r.kind != "correct":
                    tf, kw = _problem(r.kind, self.mu)
                    r.admitted = time.perf_counter()
                    in_server[self.native.submit(r.payload, self.mu, 0.0, tf, **kw)] = r
                else:
                    waiting.append(r)
            # requests the native server finished
            for rid in [q for q in in_server if self.native.poll(q) >= 2]:
                r = in_server.pop(rid)
                r.result = _native_result(r.kind, self.native.fetch(rid))
                r.done = time.perf_counter()
            # collect finished batches
            done = {f for f in futures if f.done()}
            for f in done:
                kind, reqs, sidx = f.result()
                with self.lock:
                    self.in_use -= sum(r.footprint for r in reqs)
                    self.free_streams.append(sidx)
                stats.batches += 1
            futures -= done
            # admit in arrival order while the footprint fits; merge per kind
            if waiting and self.free_streams:
                admitted, waiting, self.in_use = admit(waiting, self.in_use, self.budget, len(self.free_streams))
                for kind, reqs in admitted.items():
                    sidx = self.free_streams.pop()
                    futures.add(self.pool.submit(self._run_batch, kind, reqs, sidx))
            if not done:
                time.sleep(self.tick_s if not in_server else min(self.tick_s, 0.0005))
        stats.wall_s = time.perf_counter() - t0
        for r in requests:
            stats.n += 1
            stats.latencies.append(r.done - (t0 + r.arrival))
            if "n_accept" in r.result:
                stats.traj_steps += int(np.sum(r.result["n_accept"]))
        return stats

    def close(self):
        self.pool.shutdown(wait=True)
        if self.native is not None:
            self.native.close()
            self.native = None


def run_sequential(requests, mu, device=None, t0=None):
    """Plain form: each request alone, in arrival order, on the current stream."""
    dev = P._device(device)
    t0 = time.perf_counter() if t0 is None else t0
    stats = ServingStats()
    for r in requests:
        wait = r.arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        r.admitted = time.perf_counter()
        r.result = _solve(r.kind, r.payload, mu, dev, batched=False)
        torch.cuda.synchronize(dev)
        r.done = time.perf_counter()
        stats.n += 1
        stats.latencies.append(r.done - (t0 + r.arrival))
        if "n_accept" in r.result:
            stats.traj_steps += int(np.sum(r.result["n_accept"]))
    stats.wall_s = time.perf_counter() - t0
    return stats


def poisson_requests(rate_hz, duration_s, mu, seed=0, manifold_seeds=None, size_scale=1.0):
    """Seeded Poisson stream: kinds uniform over manifold (64-4096 seeds),
    correct (1-256 guesses) and synodic (1k-32k states), sizes log-uniform
    (multiplied by size_scale, for small test streams)."""
    from . import halo
    from . import workloads as W
    rng = np.random.default_rng(seed)
    t, rid, out = 0.0, 0, []
    if manifold_seeds is None:
        manifold_seeds = W.section_states(4096, seed=seed + 1)
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= duration_s:
            break
        kind = ("manifold", "correct", "synodic")[rng.integers(0, 3)]
        lo, hi = {"manifold": (64, 4096), "correct": (1, 256), "synodic": (1024, 32768)}[kind]
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))) * size_scale)
        n = max(1, n)
        if kind == "manifold":
            idx = rng.integers(0, len(manifold_seeds), n)
            payload = manifold_seeds[idx]
        elif kind == "correct":
            pt, az, zen = W.halo_guess_params(n, seed=int(rng.integers(1 << 30)))
            payload = np.concatenate([halo.third_order_guess(mu, int(p), a, z) for p, a, z in zip(pt, az, zen)])
        else:
            payload = W.section_states(n, seed=int(rng.integers(1 << 30)))
        out.append(Request(rid=rid, kind=kind, payload=payload, arrival=t))
        rid += 1
    return out


class NativeServer:
    """The library's native request server (``hg_serve_*``): continuous
    batching of DOP853 propagation requests behind the C ABI at the level of
    trajectory slots -- every problem (mu, dimension, span, options, event)
    gets a pool of device-resident slots that waiting requests enter as slots
    free up, segment by segment; results equal direct calls."""

    def __init__(self, device=0, hbm_budget_bytes=8 << 30, max_concurrent=4, staging_bytes=None, pool_slots=32768,
                 seg_steps=16):
        import ctypes as C
        from . import _lib
        self._C, self._lib = C, _lib
        self.L = _lib.load()
        if staging_bytes is None:
            staging_bytes = min(int(hbm_budget_bytes), 1 << 30)
        cfg = _lib.hg_serve_config(int(device), int(hbm_budget_bytes), int(max_concurrent), int(staging_bytes),
                                   int(pool_slots), int(seg_steps))
        self.ptr = C.c_void_p()
        rc = self.L.hg_serve_create(C.byref(cfg), C.byref(self.ptr))
        if rc != _lib.HG_OK:
            raise _lib.HitenGpuError(rc, "hg_serve_create failed")
        self.meta = {}

    def _check(self, rc, what):
        if rc != self._lib.HG_OK:
            raise self._lib.HitenGpuError(rc, what)

    def submit(self, y0, mu, t0, tmax, rtol=1e-12, atol=1e-12, max_step=1e4, min_step=None, max_steps=100_000,
               fwd=1, flip=None, event=None):
        C, _lib = self._C, self._lib
        y = np.ascontiguousarray(np.atleast_2d(np.asarray(y0, dtype=np.float64)))
        n, dim = y.shape
        lo, hi = P._flip(dim, fwd, flip)
        opts = _lib.hg_dop853_opts(float(rtol), float(atol), float(max_step),
                                   float(10.0 * P.EPS if min_step is None else min_step), int(max_steps), int(fwd),
                                   lo, hi)
        ev = None
        hits = 0
        if event is not None:
            hits = int(event.max_hits)
            ev = _lib.hg_event(int(event.index), float(event.offset), int(event.direction), hits,
                               float(event.xtol), float(event.gtol))
        rid = C.c_longlong(0)
        self._check(self.L.hg_serve_submit(self.ptr, float(mu), dim, n, y.ctypes.data_as(C.c_void_p), float(t0),
                                           float(tmax), C.byref(opts), C.byref(ev) if ev is not None else None,
                                           C.byref(rid)), "hg_serve_submit")
        self.meta[rid.value] = (n, dim, hits)
        return rid.value

    def poll(self, rid):
        st = self._C.c_int(0)
        self._check(self.L.hg_serve_poll(self.ptr, int(rid), self._C.byref(st)), "hg_serve_poll")
        return st.value

    def wait(self, rid, timeout=120.0):
        self._check(self.L.hg_serve_wait(self.ptr, int(rid), float(timeout)), "hg_serve_wait")

    def fetch(self, rid):
        C = self._C
        n, dim, hits = self.meta.pop(rid)
        out = {"y_end": np.empty((n, dim)), "t_end": np.empty(n), "n_accept": np.empty(n, np.int32),
               "n_reject": np.empty(n, np.int32), "status": np.empty(n, np.int32)}
        if hits:
            out.update(hit_t=np.empty((n, hits)), hit_y=np.empty((n, hits, dim)), n_hits=np.empty(n, np.int32))
        p = lambda k: out[k].ctypes.data_as(C.c_void_p) if k in out else None  # noqa: E731
        self._check(self.L.hg_serve_fetch(self.ptr, int(rid), p("y_end"), p("t_end"), p("hit_t"), p("hit_y"),
                                          p("n_hits"), p("n_accept"), p("n_reject"), p("status")), "hg_serve_fetch")
        return out

    def cancel(self, rid):
        ok = self.L.hg_serve_cancel(self.ptr, int(rid)) == self._lib.HG_OK
        if ok:
            self.meta.pop(rid, None)
        return ok

    def stats(self):
        C = self._C
        p50, p99, n, b = C.c_double(0), C.c_double(0), C.c_longlong(0), C.c_longlong(0)
        self._check(self.L.hg_serve_stats(self.ptr, C.byref(p50), C.byref(p99), C.byref(n), C.byref(b)),
                    "hg_serve_stats")
        return {"p50_ms": p50.value, "p99_ms": p99.value, "requests": n.value, "batches": b.value}

    def close(self):
        if getattr(self, "ptr", None):
            self.L.hg_serve_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
