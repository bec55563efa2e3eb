"""CUDA-graph capture of a batched DOP853 propagation.

A batch of fixed shape (N states of dimension dim, the same options and
event) is captured once as a CUDA graph of the segmented driver
(`hg_propagate_dop853_segmented`: segment set-up, `segments` compacting
launches, the deferred event refinement) over static device buffers; each
`run` copies new initial states into the static input and replays the graph.
Trajectories still running after the captured segments (status -1) are
finished by ordinary resumed calls, so results never depend on the number of
captured segments and are bit-identical to `propagate.propagate_dop853`.

Replays cost one graph launch instead of the driver's host work per segment;
the graph keeps its buffers for its lifetime (results are views of them, valid
until the next `run`).
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from . import propagate as P


class CapturedDop853:
    """Capture `propagate_dop853(y0, t0, tmax, mu, ...)` for batches of shape (n, dim)."""

    def __init__(self, n, dim, t0, tmax, mu, rtol=1e-12, atol=1e-12, max_step=1e4, min_step=None,
                 max_steps=100_000, fwd=1, flip=None, event=None, n_samples=0, sample_last_only=False,
                 seg_steps=32, segments=8, device=None):
        self.dev = P._device(device)
        self.n, self.dim = int(n), int(dim)
        if self.n < 1:
            raise ValueError("a captured batch needs at least one state")
        if np.ndim(t0) != 0 or np.ndim(tmax) != 0:
            raise ValueError("captured batches take scalar t0 and tmax")
        self.H = _lib.handle(self.dev.index or 0)
        n, d, dev = self.n, self.dim, self.dev
        lo, hi = P._flip(d, fwd, flip)
        self.opts = _lib.hg_dop853_opts(float(rtol), float(atol), float(max_step),
                                        float(10.0 * P.EPS if min_step is None else min_step), int(max_steps),
                                        int(fwd), lo, hi)
        self.event = event
        self.evp = None
        f64 = dict(dtype=torch.float64, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        self.y0 = torch.zeros((d, n), **f64)
        self.y_end = torch.zeros((d, n), **f64)
        self.t_end = torch.zeros(n, **f64)
        self.n_acc = torch.zeros(n, **i32)
        self.n_rej = torch.zeros(n, **i32)
        self.status = torch.zeros(n, **i32)
        self.hit_t = self.hit_y = self.n_hits = None
        hits = 0
        if event is not None:
            hits = int(event.max_hits)
            self.evp = _lib.hg_event(int(event.index), float(event.offset), int(event.direction), hits,
                                     float(event.xtol), float(event.gtol))
            self.hit_t = torch.full((hits, n), float("nan"), **f64)
            self.hit_y = torch.full((hits, d, n), float("nan"), **f64)
            self.n_hits = torch.zeros(n, **i32)
        self.samples = None
        if n_samples:
            rows = 1 if sample_last_only else int(n_samples)
            self.samples = torch.zeros((rows, d, n), **f64)
        self.n_samples, self.sample_last_only = int(n_samples), bool(sample_last_only)
        self.t0, self.tmax, self.mu = float(t0), float(tmax), float(mu)
        self.seg_steps, self.segments = int(seg_steps), int(segments)
        self.ws_bytes = int(self.H.lib.hg_dop853_segmented_workspace_bytes(n, d, hits))
        self.ws = torch.zeros(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.stream = torch.cuda.Stream(device=dev)
        # one plain call on the side stream first (loads the kernels, sizes the
        # handle's state), then the capture
        with torch.cuda.device(dev), torch.cuda.stream(self.stream):
            self._call(resume=0, segments=self.segments)
        self.stream.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.device(dev), torch.cuda.graph(self.graph, stream=self.stream):
            self._call(resume=0, segments=self.segments)

    def _call(self, resume, segments):
        p = P._ptr
        st = C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        self.H.check(self.H.lib.hg_propagate_dop853_segmented(
            self.H.ptr, self.mu, self.dim, self.n, p(self.y0), self.n, None, None, self.t0, self.tmax,
            C.byref(self.opts), C.byref(self.evp) if self.evp is not None else None, self.n_samples,
            1 if self.sample_last_only else 0, p(self.samples), p(self.y_end), p(self.t_end), p(self.hit_t),
            p(self.hit_y), p(self.n_hits), p(self.n_acc), p(self.n_rej), p(self.status), self.seg_steps,
            segments, resume, p(self.ws), self.ws_bytes, st))

    def run(self, y0):
        """Propagate a new batch (n, dim); returns a Dop853Result over the static buffers."""
        y = torch.as_tensor(y0, dtype=torch.float64)
        if tuple(y.shape) != (self.n, self.dim):
            raise ValueError(f"captured for shape ({self.n}, {self.dim}), got {tuple(y.shape)}")
        cur = torch.cuda.current_stream(self.dev)
        self.stream.wait_stream(cur)
        with torch.cuda.device(self.dev), torch.cuda.stream(self.stream):
            self.y0.copy_(y.to(self.dev).t())
            if self.hit_t is not None:
                self.hit_t.fill_(float("nan"))
                self.hit_y.fill_(float("nan"))
            self.graph.replay()
            # trajectories the captured segments did not finish
            while bool((self.status == _lib.HG_RUNNING).any()):
                self._call(resume=1, segments=self.segments)
        cur.wait_stream(self.stream)
        res = P.Dop853Result(y_end=self.y_end.t(), t_end=self.t_end, n_accept=self.n_acc, n_reject=self.n_rej,
                             status=self.status)
        if self.hit_t is not None:
            res.hit_t = self.hit_t.t()
            res.hit_y = self.hit_y.permute(2, 0, 1)
            res.n_hits = self.n_hits
        if self.samples is not None:
            res.samples = self.samples.permute(0, 2, 1)
        return res
