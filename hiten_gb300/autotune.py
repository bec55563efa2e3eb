"""Launch-shape autotuner.

The propagation kernels have launch-shape knobs that never change results
(lanes per 6-dim DOP853 trajectory, threads per block; see
`propagate.tuning`).  Which shape is fastest depends on the batch: a batch
that fills every SM sub-partition is throughput-bound and wants one lane per
trajectory; a small or very uneven batch is bound by its longest trajectory
and wants lane pairs, which halve the per-step latency.  `tune` times every
candidate shape on the caller's own workload with CUDA events and keeps the
fastest; results are cached per workload key for the life of the process and
optionally in a JSON file.
"""
import json
import os

import torch

from . import propagate as P

DEFAULT_SHAPES = ((1, 32), (2, 32), (1, 64), (2, 64))
_cache = {}


def _time(fn, reps):
    best = float("inf")
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def tune(key, fn, shapes=DEFAULT_SHAPES, reps=2, device=None, cache_file=None):
    """Return ((lanes_d6, block), {shape: ms}) for workload `fn` and apply the winner.

    `fn()` must run the workload once (it is called under each shape)."""
    if cache_file and not _cache and os.path.exists(cache_file):
        with open(cache_file) as f:
            _cache.update({k: tuple(v) for k, v in json.load(f).items()})
    if key in _cache:
        best = tuple(_cache[key])
        P.tuning(lanes_d6=best[0], block=best[1], device=device)
        return best, {}
    timings = {}
    for lanes, block in shapes:
        with P.tuning(lanes_d6=lanes, block=block, device=device):
            fn()  # warm
            torch.cuda.synchronize()
            timings[(lanes, block)] = _time(fn, reps)
    best = min(timings, key=timings.get)
    _cache[key] = best
    P.tuning(lanes_d6=best[0], block=best[1], device=device)
    if cache_file:
        with open(cache_file, "w") as f:
            json.dump({k: list(v) for k, v in _cache.items()}, f)
    return best, timings
