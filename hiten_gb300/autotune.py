"""Launch-shape autotuner.

The propagation kernels have launch-shape knobs that never change results
(lanes per 6-dim DOP853 trajectory, threads per block; see
`propagate.tuning`).  Which shape is fastest depends on the batch: a batch
that keeps every SM's FP64 unit busy is throughput-bound and wants one lane
per trajectory; a small or very uneven batch is bound by its longest
trajectory and wants lane pairs, which halve the per-step latency.  `tune` times every
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

# Execution plans of a 6-dim DOP853 batch: single-pass launch shapes (lanes per
# trajectory, block threads, one block per SM) and the host-scheduled driver
# (per-segment layout from the live count) with its segment length.
DOP853_PLANS = (
    {"scheduled": False, "lanes_d6": 1, "block": 32, "spread": 0},
    {"scheduled": False, "lanes_d6": 2, "block": 32, "spread": 0},
    {"scheduled": False, "lanes_d6": 2, "block": 32, "spread": 1},
    {"scheduled": False, "lanes_d6": 6, "block": 32, "spread": 0},
    {"scheduled": True, "lanes_d6": 0, "block": 32, "spread": 0, "seg_steps": 8},
    {"scheduled": True, "lanes_d6": 0, "block": 32, "spread": 0, "seg_steps": 16},
    {"scheduled": True, "lanes_d6": 0, "block": 32, "spread": 0, "seg_steps": 32},
    {"scheduled": True, "lanes_d6": 0, "block": 32, "spread": 0, "seg_steps": 16, "sm_capacity": 4.5},
    {"scheduled": True, "lanes_d6": 0, "block": 32, "spread": 0, "seg_steps": 32, "sm_capacity": 4.5},
    {"scheduled": True, "lanes_d6": 0, "block": 32, "spread": 0, "seg_steps": 48, "sm_capacity": 4.5},
    {"scheduled": True, "lanes_d6": 0, "block": 32, "spread": 0, "seg_steps": 64, "sm_capacity": 4.5},
    {"scheduled": True, "lanes_d6": 2, "block": 32, "spread": 0, "seg_steps": 16},
    {"scheduled": True, "lanes_d6": 2, "block": 32, "spread": 0, "seg_steps": 32},
)
_plan_cache = {}


def _knobs(plan):
    return {k: plan[k] for k in ("lanes_d6", "block", "spread", "seg_steps", "sm_capacity") if k in plan}


def tune_dop853(key, run, plans=DOP853_PLANS, reps=2, device=None):
    """Pick the fastest execution plan for a DOP853 workload.

    `run(scheduled)` must run the workload once.  Every plan gives the same
    bits; the winner's launch knobs are applied to the device's handle and
    the plan (with its `scheduled` flag) is returned with all timings."""
    if key in _plan_cache:
        best = _plan_cache[key]
        P.tuning(device=device, **_knobs(best))
        return best, {}
    timings = {}
    for i, plan in enumerate(plans):
        with P.tuning(device=device, **_knobs(plan)):
            run(plan["scheduled"])  # warm
            torch.cuda.synchronize()
            timings[i] = _time(lambda: run(plan["scheduled"]), reps)
    best = dict(plans[min(timings, key=timings.get)])
    _plan_cache[key] = best
    P.tuning(device=device, **_knobs(best))
    return best, {plan_name(plans[i]): ms for i, ms in timings.items()}


def plan_name(plan):
    if plan["scheduled"]:
        cap = f"_cap{plan['sm_capacity']:g}" if "sm_capacity" in plan else ""
        lanes = f"_lanes{plan['lanes_d6']}" if plan.get("lanes_d6") else ""
        return f"scheduled_seg{plan.get('seg_steps', 16)}{cap}{lanes}"
    return f"lanes{plan['lanes_d6']}_block{plan['block']}" + ("_spread" if plan.get("spread") else "")


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


# Lane layouts of the device-resident halo correction (hg_correct_halo_graph):
# lanes per 6-dim event-leg trajectory and per 42-dim STM-leg trajectory.
CORRECT_SHAPES = ((6, 12), (6, 18), (6, 14), (2, 12), (1, 12))
_correct_cache = {}


def tune_correct(key, run, shapes=CORRECT_SHAPES, reps=2, device=None):
    """Pick the lane layouts of the device corrector's legs by measurement.

    `run()` must run one correction through ``corrector.correct_halo_graph``
    (each shape rebuilds the cached graph once, in the warm-up call).  Every
    shape gives the same bits; returns the winning (lanes_d6, lanes_d42) --
    not applied to the handle, since those knobs also steer other calls: run
    the correction under ``propagate.tuning(lanes_d6=..., lanes_d42=...)`` --
    with all timings (ms)."""
    if key in _correct_cache:
        return _correct_cache[key], {}
    timings = {}
    for g6, g42 in shapes:
        with P.tuning(device=device, lanes_d6=g6, lanes_d42=g42):
            run()  # warm: builds and caches the graph for this layout
            torch.cuda.synchronize()
            timings[(g6, g42)] = _time(run, reps)
    best = min(timings, key=timings.get)
    _correct_cache[key] = best
    return best, {f"event{g6}_stm{g42}": ms for (g6, g42), ms in timings.items()}
