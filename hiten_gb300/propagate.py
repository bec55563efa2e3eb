"""Batched trajectory propagation on the GPU (FP64), the array-level API
under the reference-shaped drop-ins.

Inputs may be numpy arrays or torch tensors of shape (N, dim); results are
torch float64 CUDA tensors.  Device buffers are laid out structure-of-arrays
([dim][N]) for the kernels and exposed to callers as (..., N, dim) views.
Every call goes through ``libhitengpu.so``; there is no CPU path.
"""
import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

EPS = float(np.finfo(float).eps)
# 6-dim DOP853 batches at least this wide run as host-scheduled segments by
# default: their long tail then runs in the widest lane layout
SCHEDULE_MIN = 4096


def _device(device):
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else None
    if device is None:
        raise RuntimeError("hiten_gb300 needs a CUDA device (no CPU fallback)")
    return torch.device(device)


def _to_soa(y, dim, device):
    y = torch.as_tensor(y, dtype=torch.float64)
    if y.ndim == 1:
        y = y[None, :]
    if y.shape[-1] != dim:
        raise ValueError(f"Initial state dimension {y.shape[-1]} != system dimension {dim}")
    return y.to(device).t().contiguous()  # (dim, N)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(device):
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _flip(dim, fwd, flip):
    if flip is None:
        return 0, dim
    if isinstance(flip, slice):
        lo = 0 if flip.start is None else int(flip.start)
        hi = dim if flip.stop is None else int(flip.stop)
        return lo, hi
    lo, hi = flip
    return int(lo), int(hi)


def propagate_fixed(y0, t_vals, mu, order=8, out_every=1, fwd=1, flip=None, device=None, return_status=False):
    """Fixed-step RK (order 4/6/8) over the nodes ``t_vals`` for N states.

    Mirrors integrators/rk.py:531-588 (h_n = t_{n+1} - t_n).  Returns the
    states at nodes 0, out_every, ... as a (n_out, N, dim) tensor.
    """
    dev = _device(device)
    y0 = torch.as_tensor(y0, dtype=torch.float64)
    dim = int(y0.shape[-1])
    Y0 = _to_soa(y0, dim, dev)
    N = Y0.shape[1]
    tv = torch.as_tensor(np.ascontiguousarray(np.asarray(t_vals, dtype=np.float64))).to(dev)
    n = int(tv.numel())
    n_out = (n - 1) // int(out_every) + 1
    out = torch.empty((n_out, dim, max(N, 1)), dtype=torch.float64, device=dev)
    status = torch.zeros(max(N, 1), dtype=torch.int32, device=dev)
    lo, hi = _flip(dim, fwd, flip)
    H = _lib.handle(dev.index or 0)
    with torch.cuda.device(dev):
        H.check(H.lib.hg_propagate_fixed(H.ptr, float(mu), int(order), dim, N, _ptr(Y0), max(N, 1), _ptr(tv), n,
                                         int(out_every), _ptr(out), max(N, 1), int(fwd), lo, hi, _ptr(status),
                                         _stream(dev)))
    res = out[:, :, :N].permute(0, 2, 1)
    if return_status:
        return res, status[:N]
    return res


def propagate_fixed_event(y0, t_vals, mu, event, order=8, out_every=1, fwd=1, flip=None, device=None):
    """Fixed-step RK with a terminal plane event (integrators/rk.py:655-718).

    Returns (states (n_out, N, dim) -- rows after a crossing unwritten --,
    hit_t (N,), hit_y (N, dim), n_hits (N,))."""
    dev = _device(device)
    y0 = torch.as_tensor(y0, dtype=torch.float64)
    dim = int(y0.shape[-1])
    Y0 = _to_soa(y0, dim, dev)
    N = Y0.shape[1]
    ld = max(N, 1)
    tv = torch.as_tensor(np.ascontiguousarray(np.asarray(t_vals, dtype=np.float64))).to(dev)
    n = int(tv.numel())
    n_out = (n - 1) // int(out_every) + 1
    out = torch.full((n_out, dim, ld), float("nan"), dtype=torch.float64, device=dev)
    hit_t = torch.full((ld,), float("nan"), dtype=torch.float64, device=dev)
    hit_y = torch.full((dim, ld), float("nan"), dtype=torch.float64, device=dev)
    n_hits = torch.zeros(ld, dtype=torch.int32, device=dev)
    lo, hi = _flip(dim, fwd, flip)
    evp = _lib.hg_event(int(event.index), float(event.offset), int(event.direction), 1, float(event.xtol),
                        float(event.gtol))
    H = _lib.handle(dev.index or 0)
    with torch.cuda.device(dev):
        H.check(H.lib.hg_propagate_fixed_event(H.ptr, float(mu), int(order), dim, N, _ptr(Y0), ld, _ptr(tv), n,
                                               int(out_every), _ptr(out), ld, int(fwd), lo, hi, C.byref(evp),
                                               _ptr(hit_t), _ptr(hit_y), _ptr(n_hits), None, _stream(dev)))
    return out[:, :, :N].permute(0, 2, 1), hit_t[:N], hit_y[:, :N].t(), n_hits[:N]


@dataclass
class EventSpec:
    """Plane event g(y) = y[index] - offset (integrators/utils.py:13-123)."""

    index: int
    offset: float = 0.0
    direction: int = 0
    max_hits: int = 1
    xtol: float = 1e-12
    gtol: float = 1e-12


@dataclass
class Dop853Result:
    y_end: torch.Tensor      # (N, dim) last accepted state
    t_end: torch.Tensor      # (N,)
    n_accept: torch.Tensor   # (N,)
    n_reject: torch.Tensor
    status: torch.Tensor
    hit_t: torch.Tensor = None   # (N, max_hits)
    hit_y: torch.Tensor = None   # (N, max_hits, dim)
    n_hits: torch.Tensor = None  # (N,)
    samples: torch.Tensor = None  # (n_samples or 1, N, dim)


def propagate_dop853(y0, t0, tmax, mu, rtol=1e-12, atol=1e-12, max_step=1e4, min_step=None,
                     max_steps=100_000, fwd=1, flip=None, event=None, n_samples=0, sample_last_only=False,
                     device=None, stream=None, segmented=False, seg_steps=16, max_segments=8,
                     scheduled=None, finish=True):
    """Adaptive DOP853 for N states from t0 to tmax (scalars or (N,) arrays).

    Mirrors integrators/rk.py:2375-2549 / :2678-2803 step for step.
    ``event``: optional :class:`EventSpec`.  ``n_samples >= 2``: dense output
    at linspace(t0_i, tmax_i, n_samples) (``sample_last_only``: final sample only).
    ``segmented``: run in launches of at most ``seg_steps`` attempted steps per
    trajectory (``max_segments`` launches per asynchronous call, repeated until
    every trajectory finished), compacting the live trajectories between
    launches; results are bit-identical; ``finish=False`` returns after one
    call, the unfinished trajectories with status HG_RUNNING.  ``scheduled``: host-scheduled
    segments (``hg_propagate_dop853_scheduled``): the layout of each segment
    follows the number of trajectories still running; synchronous.  The
    default (None) schedules 6-dim batches of at least SCHEDULE_MIN states
    and runs everything else as one asynchronous launch.
    """
    dev = _device(device)
    y0 = torch.as_tensor(y0, dtype=torch.float64)
    dim = int(y0.shape[-1])
    Y0 = _to_soa(y0, dim, dev)
    N = Y0.shape[1]
    ld = max(N, 1)
    if scheduled is None:
        scheduled = (not segmented) and dim == 6 and N >= SCHEDULE_MIN
    if min_step is None:
        min_step = 10.0 * EPS
    t0a = tmaxa = None
    t0s = tmaxs = 0.0
    if np.ndim(t0) == 0:
        t0s = float(t0)
    else:
        t0a = torch.as_tensor(np.asarray(t0, dtype=np.float64)).to(dev).contiguous()
    if np.ndim(tmax) == 0:
        tmaxs = float(tmax)
    else:
        tmaxa = torch.as_tensor(np.asarray(tmax, dtype=np.float64)).to(dev).contiguous()
    lo, hi = _flip(dim, fwd, flip)
    opts = _lib.hg_dop853_opts(float(rtol), float(atol), float(max_step), float(min_step), int(max_steps),
                               int(fwd), lo, hi)
    # every entry of these is written by the kernels (per trajectory, at its
    # end or pause); the hit arrays keep NaN where no crossing was found
    y_end = torch.empty((dim, ld), dtype=torch.float64, device=dev)
    t_end = torch.empty(ld, dtype=torch.float64, device=dev)
    n_acc = torch.empty(ld, dtype=torch.int32, device=dev)
    n_rej = torch.empty(ld, dtype=torch.int32, device=dev)
    status = torch.empty(ld, dtype=torch.int32, device=dev)
    evp = None
    hit_t = hit_y = n_hits = None
    if event is not None:
        mh = int(event.max_hits)
        evp = _lib.hg_event(int(event.index), float(event.offset), int(event.direction), mh, float(event.xtol),
                            float(event.gtol))
        hit_t = torch.full((mh, ld), float("nan"), dtype=torch.float64, device=dev)
        hit_y = torch.full((mh, dim, ld), float("nan"), dtype=torch.float64, device=dev)
        n_hits = torch.empty(ld, dtype=torch.int32, device=dev)
    samples = None
    if n_samples:
        rows = 1 if sample_last_only else int(n_samples)
        samples = torch.empty((rows, dim, ld), dtype=torch.float64, device=dev)
    ws_hits = int(event.max_hits) if event is not None else 0
    H = _lib.handle(dev.index or 0)
    st = _stream(dev) if stream is None else C.c_void_p(stream)
    args = (H.ptr, float(mu), dim, N, _ptr(Y0), ld, _ptr(t0a), _ptr(tmaxa), t0s, tmaxs, C.byref(opts),
            C.byref(evp) if evp is not None else None, int(n_samples), 1 if sample_last_only else 0, _ptr(samples),
            _ptr(y_end), _ptr(t_end), _ptr(hit_t), _ptr(hit_y), _ptr(n_hits), _ptr(n_acc), _ptr(n_rej), _ptr(status))
    with torch.cuda.device(dev):
        if scheduled:
            ws_bytes = int(H.lib.hg_dop853_segmented_workspace_bytes(N, dim, ws_hits))
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
            H.check(H.lib.hg_propagate_dop853_scheduled(*args, _ptr(ws), ws_bytes, st))
        elif not segmented:
            H.check(H.lib.hg_propagate_dop853(*args, st))
        else:
            ws_bytes = int(H.lib.hg_dop853_segmented_workspace_bytes(N, dim, ws_hits))
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
            segs = int(max_segments)
            resume = 0
            while True:
                H.check(H.lib.hg_propagate_dop853_segmented(*args, int(seg_steps), segs, resume,
                                                            _ptr(ws), ws_bytes, st))
                # the caller's step budget bounds the total work; stop once no
                # trajectory is left running (or after one call: finish=False)
                if not finish or N == 0 or not bool((status[:N] == _lib.HG_RUNNING).any()):
                    break
                resume = 1
    res = Dop853Result(y_end=y_end[:, :N].t(), t_end=t_end[:N], n_accept=n_acc[:N], n_reject=n_rej[:N],
                       status=status[:N])
    if event is not None:
        res.hit_t = hit_t[:, :N].t()
        res.hit_y = hit_y[:, :, :N].permute(2, 0, 1)
        res.n_hits = n_hits[:N]
    if samples is not None:
        res.samples = samples[:, :, :N].permute(0, 2, 1)
    return res


class Dop853Batch:
    """One DOP853 call shape prepared once, for repeated batches: N states of
    dimension `dim` with the same span, options and event.  The SoA input,
    the outputs and the scheduled driver's workspace are allocated here; each
    `run(y0)` copies the new states in (one transpose copy), resets the hit
    arrays to NaN (one fill: they share one buffer), and calls the library --
    the host work of `propagate_dop853` (argument handling, allocations, size
    queries, result views) is done once.  Results are the same bits as
    `propagate_dop853` with the same arguments; `run` returns one
    Dop853Result whose tensors are views of the batch's buffers, valid until
    the next `run`.  The outputs share one device arena, so `to_host()` reads
    all of them back in a single copy.  Scalar t0 / tmax; no dense samples."""

    def __init__(self, n, dim, t0, tmax, mu, rtol=1e-12, atol=1e-12, max_step=1e4, min_step=None,
                 max_steps=100_000, fwd=1, flip=None, event=None, scheduled=None, device=None):
        if np.ndim(t0) != 0 or np.ndim(tmax) != 0:
            raise ValueError("a prepared batch takes scalar t0 and tmax")
        self.dev = _device(device)
        if self.dev.index is None:
            self.dev = torch.device("cuda", torch.cuda.current_device())
        self.n, self.dim = int(n), int(dim)
        if self.n < 1:
            raise ValueError("a prepared batch needs at least one state")
        self.scheduled = ((self.dim == 6 and self.n >= SCHEDULE_MIN) if scheduled is None else bool(scheduled))
        n, d, ld, dev = self.n, self.dim, self.n, self.dev
        self.Y0 = torch.empty((d, ld), dtype=torch.float64, device=dev)
        self.stage = None  # (N, dim) device copy of host inputs, made on the first host run
        mh = int(event.max_hits) if event is not None else 0
        # the outputs, carved from one arena
        self.layout = self.arena_layout(d, ld, mh)
        nbytes = sum(self.part_bytes(dt, shape) for _, dt, shape in self.layout)
        self.out = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        self.out_host = None  # pinned mirror of the arena, made on the first to_host()
        v = self._carve(self.out)
        self.y_end, self.t_end, self.n_acc, self.n_rej, self.status = (v["y_end"], v["t_end"], v["n_acc"],
                                                                        v["n_rej"], v["status"])
        lo, hi = _flip(d, fwd, flip)
        self.opts = _lib.hg_dop853_opts(float(rtol), float(atol), float(max_step),
                                        float(10.0 * EPS if min_step is None else min_step), int(max_steps),
                                        int(fwd), lo, hi)
        self.evp = None
        self.hits = None
        if event is not None:
            self.evp = _lib.hg_event(int(event.index), float(event.offset), int(event.direction), mh,
                                     float(event.xtol), float(event.gtol))
            self.hits = v["hits"]
            hit_t = self.hits[:mh * ld].view(mh, ld)
            hit_y = self.hits[mh * ld:].view(mh, d, ld)
            self.n_hits = v["n_hits"]
        self.H = _lib.handle(dev.index or 0)
        self.ws_bytes = int(self.H.lib.hg_dop853_segmented_workspace_bytes(n, d, mh)) if self.scheduled else 0
        self.ws = torch.empty(max(self.ws_bytes, 1), dtype=torch.uint8, device=dev) if self.scheduled else None
        self.args = (self.H.ptr, float(mu), d, n, _ptr(self.Y0), ld, None, None, float(t0), float(tmax),
                     C.byref(self.opts), C.byref(self.evp) if self.evp is not None else None, 0, 0, None,
                     _ptr(self.y_end), _ptr(self.t_end), _ptr(hit_t) if mh else None,
                     _ptr(hit_y) if mh else None, _ptr(self.n_hits) if mh else None, _ptr(self.n_acc),
                     _ptr(self.n_rej), _ptr(self.status))
        self.mh = mh
        self.result = self._result(v)
        self.result_host = None

    @staticmethod
    def arena_layout(dim, n, max_hits):
        """(name, dtype, shape) of the output parts in arena order: float64
        parts first, then int32; the hits part holds hit_t then hit_y (one
        NaN fill per run)."""
        lay = [("y_end", torch.float64, (dim, n)), ("t_end", torch.float64, (n,))]
        if max_hits:
            lay.append(("hits", torch.float64, (max_hits * n * (1 + dim),)))
        lay += [("n_acc", torch.int32, (n,)), ("n_rej", torch.int32, (n,)), ("status", torch.int32, (n,))]
        if max_hits:
            lay.append(("n_hits", torch.int32, (n,)))
        return lay

    @staticmethod
    def part_bytes(dtype, shape):
        """Bytes a part takes in the arena: its size rounded up to 8, so that
        every part starts 8-byte aligned."""
        return ((math.prod(shape) * (8 if dtype == torch.float64 else 4) + 7) // 8) * 8

    def _carve(self, buf):
        """The named output parts as views of the byte buffer `buf` (the
        device arena or its pinned host mirror)."""
        views, off = {}, 0
        for name, dt, shape in self.layout:
            size = math.prod(shape) * (8 if dt == torch.float64 else 4)
            views[name] = buf[off:off + size].view(dt).view(shape)
            off += self.part_bytes(dt, shape)
        return views

    def _result(self, v):
        n, d = self.n, self.dim
        r = Dop853Result(y_end=v["y_end"].t(), t_end=v["t_end"], n_accept=v["n_acc"], n_reject=v["n_rej"],
                         status=v["status"])
        if self.mh:
            r.hit_t = v["hits"][:self.mh * n].view(self.mh, n).t()
            r.hit_y = v["hits"][self.mh * n:].view(self.mh, d, n).permute(2, 0, 1)
            r.n_hits = v["n_hits"]
        return r

    def to_host(self):
        """The last run's results on the host: one device-to-host copy of the
        output arena into pinned memory (allocated on the first call), after
        the run on the current stream.  Returns a Dop853Result of CPU tensors
        that view that memory, valid until the next `to_host`."""
        if self.out_host is None:
            self.out_host = torch.empty(self.out.numel(), dtype=torch.uint8, pin_memory=True)
            self.result_host = self._result(self._carve(self.out_host))
        self.out_host.copy_(self.out, non_blocking=True)
        torch.cuda.current_stream(self.dev).synchronize()
        return self.result_host

    def run(self, y0):
        """Propagate the (N, dim) states `y0` (a CUDA tensor on the batch's
        device, or anything torch.as_tensor takes)."""
        y = torch.as_tensor(y0, dtype=torch.float64)
        if tuple(y.shape) != (self.n, self.dim):
            raise ValueError(f"prepared for shape ({self.n}, {self.dim}), got {tuple(y.shape)}")
        if y.device != self.dev:
            # host states: one contiguous copy (asynchronous from pinned memory), then the transpose on the device
            if self.stage is None:
                self.stage = torch.empty((self.n, self.dim), dtype=torch.float64, device=self.dev)
            self.stage.copy_(y, non_blocking=bool(y.is_pinned()))
            y = self.stage
        self.Y0.copy_(y.t())
        if self.hits is not None:
            self.hits.fill_(float("nan"))
        if torch.cuda.current_device() != self.dev.index:
            with torch.cuda.device(self.dev):
                self._call()
        else:
            self._call()
        return self.result

    def _call(self):
        st = _stream(self.dev)
        if self.scheduled:
            self.H.check(self.H.lib.hg_propagate_dop853_scheduled(*self.args, _ptr(self.ws), self.ws_bytes, st))
        else:
            self.H.check(self.H.lib.hg_propagate_dop853(*self.args, st))


def fp64_peak_tflops(device=None):
    """Measured FP64 FMA throughput of the device (TFLOP/s)."""
    dev = _device(device)
    H = _lib.handle(dev.index or 0)
    v = C.c_double(0.0)
    with torch.cuda.device(dev):
        H.check(H.lib.hg_probe_fp64_peak(H.ptr, C.byref(v)))
    return v.value


class tuning:
    """Set the launch shape of the device's handle (results are unchanged):
    ``lanes_d6`` in {0 (auto), 1, 2, 6} lanes per 6-dim DOP853 trajectory,
    ``block`` in {32, 64, 128} threads per block, ``seg_steps`` attempted
    steps per segment of the scheduled driver, ``spread`` one 4-warp block
    per SM for DOP853, ``lanes_d42`` in {0 (auto), 7, 14, 12 (paired warps), 18 (three warps)} lanes per 42-dim
    trajectory, ``sm_capacity`` the warps an SM serves at full speed in the
    layout cost models (a float, default 3.0), ``refine_pool_mb`` the largest
    crossing-record pool of a single-pass call (larger ones refine inline).  Usable as a context manager
    (restores the previous values on exit) or as a plain call."""

    _KEYS = (("lanes_d6", _lib.HG_TUNE_DOP853_LANES_D6), ("block", _lib.HG_TUNE_BLOCK_THREADS),
             ("seg_steps", _lib.HG_TUNE_SEG_STEPS), ("spread", _lib.HG_TUNE_SPREAD),
             ("lanes_d42", _lib.HG_TUNE_LANES_D42), ("sm_capacity", _lib.HG_TUNE_SM_CAPACITY),
             ("refine_pool_mb", _lib.HG_TUNE_REFINE_POOL_MB))

    def __init__(self, lanes_d6=None, block=None, device=None, seg_steps=None, spread=None, lanes_d42=None,
                 sm_capacity=None, refine_pool_mb=None):
        dev = _device(device)
        self.H = _lib.handle(dev.index or 0)
        self.old = {k: self.H.get_tuning(key) for k, key in self._KEYS}
        new = {"lanes_d6": lanes_d6, "block": block, "seg_steps": seg_steps,
               "spread": None if spread is None else int(bool(spread)), "lanes_d42": lanes_d42,
               "sm_capacity": None if sm_capacity is None else int(round(10 * sm_capacity)),
               "refine_pool_mb": refine_pool_mb}
        for k, key in self._KEYS:
            if new[k] is not None:
                self.H.set_tuning(key, new[k])

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        for k, key in self._KEYS:
            self.H.set_tuning(key, self.old[k])
