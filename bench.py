#!/usr/bin/env python
"""Benchmark: batched adaptive DOP853 manifold propagation (FP64).

Workload (one "step" = one pass of the hot path over the whole batch):
stable manifold of the Earth-Moon (mu = 0.012150585609624) L1 southern halo
with Az = 0.2 (x0, T as corrected by the reference): 512 phases x 32
displacements log-uniform in [1e-7, 1e-5] along the stable eigenvector =
16384 trajectories, DOP853 rtol = atol = 1e-12, integrated backward to
t = -8 with a terminal event on the plane x = 1 - mu (uneven lengths).
Seeds are synthetic (seeded), computed on the GPU from the orbit's STM grid.
The execution plan -- one persistent lane-refill launch with a given lane
layout, or host-scheduled segments that compact the live trajectories and
widen the layout as they thin out -- is chosen by the autotuner on this
workload (every plan gives the same bits).

Metric: accepted trajectory-steps per second (attempted steps reported
beside it).  `value`: throughput with the seeds resident in HBM, each step
one run of the call prepared once (propagate.Dop853Batch: static input,
output and workspace buffers; checked bit-identical to propagate_dop853);
`e2e`: the same prepared call from pinned host seeds, the H2D copy of the
seeds and the D2H copy of every output (the batch's output arena, one copy:
Dop853Batch.to_host) inside the timed region (wall clock); `e2e.dropin` the
same through the
reference-shaped public API (hiten_gb300.manifold.propagate_to_plane, a full
per-call setup).  `gpu_launches`:
kernels launched in the timed region, read from the library's counter.

`secondary`: the other workloads of the metric, measured in the same run
after the headline -- fixed-step RK8 with the STM (1024 states x 3000 steps),
the synodic section (65536 states, <= 8 crossings), batched halo correction
(2048 guesses, ||r|| and ||dx||) and the serving mix (Poisson 200 req/s,
p50/p99) -- each with its time, roofline fraction of the FP64 peak, plain-GPU
form and CPU oracle baseline (`--no-secondary` skips them; `--workload W`
runs one alone).

`--impl reference`: the reference's algorithm on the host cores (the CPU
oracle in numba-lowering mode, one trajectory per task, all host threads),
on a bounded sample of the same seeds.
"""
import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "FP64 trajectory-steps/sec w/ STM (batched/served vs plain GPU vs CPU); p50/p99 latency"
UNIT = "traj-steps/s"
# algorithmic flops of one attempted DOP853 step at d = 6 (add/mul = 1, FMA = 2,
# div = sqrt = 1): 12 right-hand sides x 31 + 2 (50 + 8) 6 stage sums
# + 2 (8 + 8) 6 error estimates + 9 x 6 error norm
FLOPS_PER_ATTEMPT_D6 = 1314.0
N_PHASE, N_DISP = 512, 32
TF = 8.0


def config(n_gpus):
    return {"workload": "manifold.compute: L1 halo Az=0.2 stable manifold, 512 phases x 32 displacements "
                        "(16384 trajectories), DOP853 rtol=atol=1e-12 to t=-8, terminal event x=1-mu",
            "trajectories_per_gpu": N_PHASE * N_DISP, "dim": 6, "rtol": 1e-12,
            "parallelism": f"replicas x{n_gpus}", "l2": "flushed between timed steps (256 MiB write)"}


def sched_lanes(n_live, warp_slots):
    """Lanes per trajectory the scheduled DOP853 driver gives a segment of
    n_live trajectories: the least of lat(G) x max(1, warps / warp_slots)
    (the same rule as the library's)."""
    best, best_cost = 1, None
    for g, per_warp, lat in ((1, 32, 1.0), (2, 16, 0.622), (6, 5, 0.400)):
        cost = lat * max(1.0, -(-n_live // per_warp) / warp_slots)
        if best_cost is None or cost < best_cost:
            best, best_cost = g, cost
    return best


def dominant_launch(run_segment, plan, n, sm_count, stream, reps=3):
    """The step's dominant kernel launch timed alone (CUDA events on its
    stream, inside the NVTX range "dominant_launch" so that a profiler can
    capture the same launch): for a scheduled plan its first segment, every
    trajectory live, in the layout the driver's rule gives n trajectories and
    the plan's segment length.  Returns (lanes, ms, attempted steps) or None
    for a single-pass plan (whose one launch is the step)."""
    import torch
    if not plan.get("scheduled"):
        return None
    g = plan.get("lanes_d6") or sched_lanes(n, plan.get("sm_capacity", 3.0) * sm_count)
    seg = int(plan.get("seg_steps", 16))
    run_segment(g, seg)  # warm
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms, att = [], 0
    torch.cuda.nvtx.range_push("dominant_launch")
    for _ in range(reps):
        torch.cuda.synchronize()
        # a bounded device sleep (~1 ms) while the host enqueues the call, so
        # that the events time the device work, not the host's issue latency
        if hasattr(torch.cuda, "_sleep"):  # private; without it the host latency stays in
            torch.cuda._sleep(2_000_000)
        e0.record(stream)
        r = run_segment(g, seg)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        att = int((r.n_accept + r.n_reject).sum().item())
    torch.cuda.nvtx.range_pop()
    return g, statistics.median(ms), att


def make_seeds(device):
    from hiten_gb300 import manifold as M
    from hiten_gb300 import workloads as W
    mu = W.MU_EM
    times, PHI = M.stm_grid(W.HALO_L1_AZ02_X0, W.HALO_L1_AZ02_T, mu, steps=2000, forward=-1, device=device)
    v = M.stable_eigvec(PHI[-1, :36].reshape(6, 6), stable=True)
    phases, disp = W.manifold_grid(N_PHASE, N_DISP, seed=0)
    return M.seeds(times, PHI, W.HALO_L1_AZ02_T, phases, disp, v, direction=1)


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region.

    The sampler is started before the warm-up steps (nvidia-smi's own start-up queries the driver
    heavily, which delays the host calls of a synchronous driver if it falls inside the timed region);
    `begin()` / `end()` mark the timed region on the host clock and `summary()` keeps the samples
    taken inside it (the nearest one on either side as well, so that a short region has samples)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    INTERVAL_MS = 200

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.t_begin = self.t_end = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def begin(self):
        self.t_begin = time.time()

    def end(self):
        self.t_end = time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    @staticmethod
    def _stamp(text):
        import datetime
        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.datetime.strptime(text, fmt).timestamp()
            except ValueError:
                pass
        return None

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = []
        for line in self.f.read().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 10:
                continue
            try:
                rows.append((self._stamp(p[0]), float(p[2]), float(p[3]), p[6:10]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        if rows and self.t_begin is not None and self.t_end is not None and all(r[0] is not None for r in rows):
            inside = [r for r in rows if self.t_begin <= r[0] <= self.t_end]
            before = [r for r in rows if r[0] < self.t_begin][-1:]
            after = [r for r in rows if r[0] > self.t_end][:1]
            rows = before + inside + after
        sm = [r[1] for r in rows]
        mx = [r[2] for r in rows]
        reasons = set()
        for r in rows:
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), r[3]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference(seeds, sample, threads, mode_name="NUMBA", min_seconds=3.0):
    """Time the CPU oracle (reference algorithm) on `sample` seeds with all threads, repeating the
    sample until at least `min_seconds` of wall time are covered."""
    from oracle import hgo
    from hiten_gb300 import workloads as W
    mu = W.MU_EM
    hgo.set_mode(getattr(hgo, "MODE_" + mode_name))
    s = seeds[:sample]
    acc = 0
    t0 = time.perf_counter()
    while True:  # repeat the sample until the timing covers at least min_seconds
        r = hgo.dop853_event_batch(s, 0.0, TF, mu, 0, 1 - mu, 0, 1, max_step=1e4, fwd=-1, flip=(0, 6),
                                   threads=threads)
        acc += int(r["n_accept"].sum())
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    return float(acc) / dt, dt, acc


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from hiten_gb300 import manifold as M
    from hiten_gb300 import workloads as W
    from oracle import hgo
    # the same seeds as the GPU arm: the orbit's STM grid from the oracle
    # (DEVICE mode is bit-identical to the GPU kernel), host seeding code
    hgo.set_mode(hgo.MODE_DEVICE)
    T = W.HALO_L1_AZ02_T
    PHI, _, _, _ = hgo.dop853_dense(W.identity_stm_state(W.HALO_L1_AZ02_X0)[0], np.linspace(0.0, T, 2000), W.MU_EM,
                                    fwd=-1, flip=(36, 42))
    v = M.stable_eigvec(PHI[-1, :36].reshape(6, 6), stable=True)
    phases, disp = W.manifold_grid(N_PHASE, N_DISP, seed=0)
    seeds = M.seeds(-np.linspace(0.0, T, 2000), PHI, T, phases, disp, v, direction=1)
    threads = os.cpu_count() or 1
    sample = len(seeds)
    vals = []
    for i in range(args.warmup + args.steps):
        v, dt, n = cpu_reference(seeds, sample, threads, min_seconds=2.0)
        if i >= args.warmup:
            vals.append((v, dt))
    value = statistics.median(v for v, _ in vals)
    ms = statistics.median(dt for _, dt in vals) * 1e3
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": config(args.gpus),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"all {sample} manifold seeds per step, repeated to >= 2 s (CPU oracle, "
                                      f"numba lowering of powers, libm pow), one trajectory per task"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def whole_job_rate(local_units, local_seconds, device=None):
    """(units of all ranks / the slowest rank's seconds, that time).  Ranks are
    replicas with no data-path exchange; only these two numbers cross ranks."""
    import torch
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
        s = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        dist.all_reduce(s, op=dist.ReduceOp.MAX)
        return float(u.item()) / float(s.item()), float(s.item())
    return float(local_units) / float(local_seconds), float(local_seconds)


def _event_ms(fn, reps):
    import torch
    fn()
    torch.cuda.synchronize()
    ts, r = [], None
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        r = fn()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts), r


def _line(name, metric, value, unit, ms, cfg, **extra):
    out = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "ms_per_step": ms, "higher_is_better": True,
           "dtype": "f64", "data": "synthetic", "config": dict(workload=name, **cfg)}
    out.update(extra)
    print(json.dumps(out))


def _print_secondary(d):
    """One JSON line for a secondary workload run on its own (--workload)."""
    extra = {k: v for k, v in d.items() if k not in ("workload", "metric", "value", "unit", "ms", "config")}
    _line(d["workload"], d["metric"], d["value"], d["unit"], d["ms"], d.get("config", {}), **extra)


def _roofline(flops, ms, peak, note):
    achieved = flops / (ms * 1e-3) / 1e12
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if peak else None, "flops": flops, "work": note,
            "peak_source": "measured: DFMA throughput probe (hg_probe_fp64_peak) on this GPU"}


def _cpu_loop(fn, min_seconds):
    """Repeat fn() (returning units of work) until min_seconds of wall time; (units/s, seconds, units)."""
    units = 0
    t0 = time.perf_counter()
    while True:
        units += fn()
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            return units / dt, dt, units


def _peak(dev):
    from hiten_gb300 import propagate as P
    return P.fp64_peak_tflops(dev)


FLOPS_PER_STEP_RK8_D42 = 7870.0
FLOPS_PER_ATTEMPT_D42 = 8586.0


def sec_fixed_stm(steps, dev, peak, cpu=True):
    """Fixed-step RK8 with the 42-dim variational system, 1024 states (STM = I),
    t in [0, 3], 3000 steps, every 100th state written."""
    import torch
    from hiten_gb300 import propagate as P
    from hiten_gb300 import workloads as W
    y_host = W.stm_fixed_batch(1024, seed=0)
    y = torch.as_tensor(y_host, device=dev)
    t = np.linspace(0.0, 3.0, 3001)
    ms, _ = _event_ms(lambda: P.propagate_fixed(y, t, W.MU_EM, order=8, out_every=100, device=dev), max(3, steps // 4))
    units = 1024 * 3000
    n_plain = 8
    pms, _ = _event_ms(lambda: [P.propagate_fixed(y[i:i + 1], t, W.MU_EM, order=8, out_every=100, device=dev)
                                for i in range(n_plain)], 1)
    out = {"workload": "RK8 + STM, 1024 states x 3000 steps (42-dim)", "metric": METRIC,
           "value": units / (ms * 1e-3), "unit": UNIT, "ms": ms, "config": {"states": 1024, "steps": 3000, "dim": 42},
           "timing": "CUDA events on the launching stream, median",
           "roofline": _roofline(FLOPS_PER_STEP_RK8_D42 * units, ms, peak, "7870 flops per 42-dim RK8 step"),
           "plain_gpu": {"value": n_plain * 3000 / (pms * 1e-3), "unit": UNIT,
                         "form": f"one call per trajectory, {n_plain}-trajectory sample"}}
    if cpu:
        from oracle import hgo
        hgo.set_mode(hgo.MODE_NUMBA)
        th = os.cpu_count() or 1
        v, dt, n = _cpu_loop(lambda: (hgo.fixed_rk_batch(8, y_host, t, W.MU_EM, out_every=100, threads=th), 1024 * 3000)[1],
                             2.0)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": th, "kind": "port",
                               "sample": f"all 1024 states x 3000 steps, repeated: {n} steps in {dt:.1f} s "
                                         f"(CPU oracle, numba lowering of powers, libm pow)"}
    return out


def bench_fixed_stm(args):
    import torch
    dev = torch.device("cuda", 0)
    _print_secondary(sec_fixed_stm(args.steps, dev, _peak(dev), cpu=not args.no_cpu_baseline))


def sec_section(steps, dev, peak, cpu=True):
    """Synodic section: 65536 Jacobi-matched states near L1/L2, DOP853 1e-11 to t = 20, up to 8 y = 0
    crossings (direction -1) each; the execution plan (single pass or host-scheduled segments, same bits)
    chosen by the autotuner on this workload."""
    import torch
    from hiten_gb300 import autotune
    from hiten_gb300 import propagate as P
    from hiten_gb300 import workloads as W
    y_host = W.section_states(65536, seed=0)
    y = torch.as_tensor(y_host, device=dev)
    ev = P.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)

    def run(scheduled, yy=y):
        return P.propagate_dop853(yy, 0.0, 20.0, W.MU_EM, rtol=1e-11, atol=1e-11, event=ev, device=dev,
                                  scheduled=scheduled)

    plan, plan_ms = autotune.tune_dop853("section_65536", run, device=dev)
    ms, r = _event_ms(lambda: run(plan["scheduled"]), max(2, steps // 4))
    acc, att = int(r.n_accept.sum()), int(r.n_accept.sum() + r.n_reject.sum())
    n_plain = 16
    plain = []
    pms, _ = _event_ms(lambda: plain.extend(run(False, y[i:i + 1]) for i in range(n_plain)), 1)
    plain_acc = sum(int(x.n_accept.sum()) for x in plain[-n_plain:])
    out = {"workload": "synodic section, 65536 states, DOP853 1e-11 to t=20, <= 8 crossings", "metric": METRIC,
           "value": acc / (ms * 1e-3), "unit": UNIT, "ms": ms,
           "config": {"states": 65536, "max_hits": 8, "plan": autotune.plan_name(plan)},
           "timing": "CUDA events on the launching stream, median (the scheduled driver reads the live count "
                     "back between segments inside the timed region)",
           "attempted_steps_per_s": att / (ms * 1e-3), "autotune_ms": plan_ms,
           "mean_hits": float(r.n_hits.float().mean()),
           "roofline": _roofline(FLOPS_PER_ATTEMPT_D6 * att, ms, peak, "1314 flops per attempted 6-dim DOP853 step"),
           "plain_gpu": {"value": plain_acc / (pms * 1e-3), "unit": UNIT,
                         "form": f"one single-pass call per trajectory, {n_plain}-trajectory sample"}}
    if cpu:
        from oracle import hgo
        hgo.set_mode(hgo.MODE_NUMBA)
        th = os.cpu_count() or 1
        sub = y_host[np.random.default_rng(1).choice(len(y_host), 1024, replace=False)]

        def one():
            rr = hgo.dop853_event_batch(sub, 0.0, 20.0, W.MU_EM, 1, 0.0, -1, 8, rtol=1e-11, atol=1e-11, max_step=1e4,
                                        threads=th)
            return int(rr["n_accept"].sum())
        v, dt, n = _cpu_loop(one, 2.0)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": th, "kind": "port",
                               "sample": f"1024 seeded states of the 65536, repeated: {n} accepted steps in "
                                         f"{dt:.1f} s (CPU oracle, numba lowering, libm pow)"}
    return out


def bench_section(args):
    import torch
    dev = torch.device("cuda", 0)
    _print_secondary(sec_section(args.steps, dev, _peak(dev), cpu=not args.no_cpu_baseline))


def bench_synodic_detect(args):
    """Sample-based synodic crossing detection (SynodicMap.compute on sampled trajectories): 65536 section
    states propagated by DOP853 1e-11 with dense output at 301 samples over t in [0, 3] (a step budget of 3000
    stops the few states that graze a primary), then the detection kernel on the samples: y = 0, direction -1,
    plane (x, vx), 50-fold segment refinement, Newton <= 10, <= 8 hits, cubic and linear interpolation.
    The value is sample segments scanned per second (cubic)."""
    import torch
    from hiten_gb300 import propagate as P
    from hiten_gb300 import synodic as S
    from hiten_gb300 import workloads as W
    dev = torch.device("cuda", 0)
    n, m = 65536, 301
    y = torch.as_tensor(W.section_states(n, seed=0), device=dev)
    times = torch.linspace(0.0, 3.0, m, dtype=torch.float64, device=dev)
    r = P.propagate_dop853(y, 0.0, 3.0, W.MU_EM, rtol=1e-11, atol=1e-11, max_step=1e4, max_steps=3000,
                           n_samples=m, device=dev)
    res = {}
    for interp in ("cubic", "linear"):
        def det():
            return S.detect(times, r.samples, section_axis="y", section_offset=0.0, plane_coords=("x", "vx"),
                            direction=-1, segment_refine=50, interp=interp, newton_max_iter=10, max_hits=8,
                            device=dev)
        ms, (ht, hy, nh) = _event_ms(det, max(3, args.steps // 2))
        res[interp] = (ms, float(nh.float().mean()))
    ms, hits = res["cubic"]
    segs = n * (m - 1)
    sample_bytes = m * 2 * n * 8  # the scan reads y and vy (value and slope of the section function)
    _line("synodic detection on samples, 65536 states x 301 samples (cubic, 50-fold refinement)",
          "section segments scanned/s", segs / (ms * 1e-3), "segments/s", ms,
          {"states": n, "samples": m, "segment_refine": 50, "interp": "cubic", "max_hits": 8},
          mean_hits=hits, linear={"ms": res["linear"][0], "mean_hits": res["linear"][1]},
          roofline={"bound": "fp64", "bytes_read": sample_bytes, "achieved_gbs": sample_bytes / (ms * 1e-3) / 1e9,
                    "fp64_pipe_active": 0.835, "dram_throughput": 0.004,
                    "source": "ncu of section_kernel on this workload (profiles/section_kernel_synodic_65536.md): "
                              "the cubic Hermite evaluations and refinements hold the FP64 pipe; the scanned "
                              "components are read once"})


def sec_correct(steps, dev, peak, cpu=True):
    """Batched halo correction: 2048 third-order guesses (half L1, half L2,
    Az ~ U[0.01, 0.4], zenith 50/50 seeded), single shooting on the half-period y = 0 crossing until
    ||r||_inf < 1e-12 (the reference's criterion); ||dx||_inf of one more Newton step at the result is
    reported beside it."""
    import torch
    from hiten_gb300 import corrector, halo
    from hiten_gb300 import workloads as W
    mu = W.MU_EM
    pt, az, zen = W.halo_guess_params(2048, seed=0)
    g = np.concatenate([halo.third_order_guess(mu, 1, az[pt == 1], zen[pt == 1]),
                        halo.third_order_guess(mu, 2, az[pt == 2], zen[pt == 2])])
    corrector.correct_halo_native(g[:64], mu)
    torch.cuda.synchronize()
    reps = max(2, steps // 4)
    # the device-resident form: every orbit's Newton iterations and line
    # searches inside one CUDA graph (built on the first call, then replayed)
    from hiten_gb300 import _lib
    L = _lib.load()
    ws = torch.empty(int(L.hg_correct_halo_graph_workspace_bytes(len(g))) + 256, dtype=torch.uint8, device=dev)
    from hiten_gb300 import autotune
    from hiten_gb300 import propagate as P
    shape, shape_ms = autotune.tune_correct("correct_2048", lambda: corrector.correct_halo_graph(g, mu, workspace=ws),
                                            device=dev)
    tg = []
    with P.tuning(device=dev, lanes_d6=shape[0], lanes_d42=shape[1]):
        gr = corrector.correct_halo_graph(g, mu, workspace=ws)  # (re)builds the graph for the chosen layout
        torch.cuda.synchronize()
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            gr = corrector.correct_halo_graph(g, mu, workspace=ws)
            torch.cuda.synchronize()
            tg.append(time.perf_counter() - t0)
    sg = statistics.median(tg)
    tn = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nat = corrector.correct_halo_native(g, mu)
        torch.cuda.synchronize()
        tn.append(time.perf_counter() - t0)
    sn = statistics.median(tn)
    # the Python host loop over the same kernels, with its attempted-step count for the roofline
    be = corrector.GpuShootingBackend(mu, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = corrector.correct_halo(g, mu, backend=be)
    torch.cuda.synchronize()
    sp = time.perf_counter() - t0
    flops = FLOPS_PER_ATTEMPT_D6 * be.attempts[6] + FLOPS_PER_ATTEMPT_D42 * be.attempts[42]
    ok = gr.status == 0
    dx = corrector.newton_step_norms(gr.x0[ok], mu, device=dev)
    both = ok & (nat.status == 0)
    n_plain = 8
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(n_plain):
        corrector.correct_halo(g[i:i + 1], mu)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    out = {"workload": "halo correction, 2048 guesses (L1/L2, Az 0.01-0.4)", "metric": "orbits corrected/s",
           "value": len(g) / sg, "unit": "orbits/s", "ms": sg * 1e3,
           "config": {"orbits": len(g), "driver": "hg_correct_halo_graph (one CUDA graph per correction)",
                      "zenith": "seeded 50/50"},
           "timing": "host wall clock around the call and a device synchronize (the graph replays; inputs copied "
                     "in and results out inside), median",
           "graph": {"host_launch_calls_per_correction": int(gr.launches),
                     "layout": {"event_lanes": shape[0], "stm_lanes": shape[1], "autotune_ms": shape_ms},
                     "same_status_as_host_driver": int(np.sum(gr.status == nat.status)),
                     "max_state_diff_vs_host_driver": float(np.max(np.abs(gr.x0[both] - nat.x0[both]))),
                     "max_period_diff_vs_host_driver": float(np.max(np.abs(gr.period[both] - nat.period[both]))),
                     "iterations_diff_max": int(np.max(np.abs(gr.iterations - nat.iterations)))},
           "native_host_driver": {"ms": sn * 1e3, "orbits_per_s": len(g) / sn,
                                  "converged": int((nat.status == 0).sum())},
           "converged": int(ok.sum()), "iterations_hist": np.bincount(gr.iterations).tolist(),
           "convergence": {"residual_inf_max": float(np.max(gr.residual_norm[ok])),
                           "dx_inf_max": float(np.nanmax(dx)), "dx_inf_median": float(np.nanmedian(dx)),
                           "dx_below_1e-12": int(np.sum(dx < 1e-12)),
                           "criterion": "stop when ||r||_inf < 1e-12 (the reference's test); ||dx||_inf is the "
                                        "next Newton correction at the corrected state"},
           "roofline": _roofline(flops, sp * 1e3, peak,
                                 f"Python host loop over the same kernels: {be.attempts[6]} attempted 6-dim steps "
                                 f"x 1314 + {be.attempts[42]} attempted 42-dim steps x 8586 flops, over its "
                                 f"wall time {sp * 1e3:.1f} ms (legs are latency-bound)"),
           "python_host_loop": {"ms": sp * 1e3, "orbits_per_s": len(g) / sp, "converged": int((res.status == 0).sum()),
                                "gpu_launches": res.launches},
           "plain_gpu": {"value": n_plain / plain_s, "unit": "orbits/s",
                         "form": f"one correction call per orbit, {n_plain}-orbit sample"}}
    if cpu:
        from oracle import hgo
        from oracle.shooting import OracleShootingBackend
        th = os.cpu_count() or 1
        sub = g[:32]
        v, dt, n = _cpu_loop(lambda: int(np.sum(corrector.correct_halo(
            sub, mu, backend=OracleShootingBackend(hgo, mu, hgo.MODE_NUMBA, threads=th)).status >= 0)), 2.0)
        out["cpu_baseline"] = {"value": v, "unit": "orbits/s", "cores": th, "kind": "port",
                               "sample": f"32 of the guesses, repeated: {n} corrections in {dt:.1f} s (the same "
                                         f"Newton/Armijo host loop over the CPU oracle's propagations, numba lowering; "
                                         f"event legs threaded, STM legs one orbit at a time)"}
    return out


def bench_correct(args):
    import torch
    dev = torch.device("cuda", 0)
    _print_secondary(sec_correct(args.steps, dev, _peak(dev), cpu=not args.no_cpu_baseline))


def sec_serving(steps, dev, peak, cpu=True, seeds=None):
    """Serving mix: seeded Poisson stream (200 req/s for 1 s) of manifold (64-4096 seeds), correction
    (1-256 guesses) and synodic (1k-32k states) requests; continuous batching vs the same stream run
    sequentially in the plain form (one single-pass call per request)."""
    from hiten_gb300 import serving
    from hiten_gb300 import workloads as W
    mu = W.MU_EM
    if seeds is None:
        seeds = make_seeds(dev)
    serving.run_sequential(serving.poisson_requests(200.0, 0.05, mu, seed=2, manifold_seeds=seeds,
                                                    size_scale=0.05), mu)

    def stream(burst=False):
        reqs = serving.poisson_requests(200.0, 1.0, mu, seed=1, manifold_seeds=seeds)
        if burst:  # every request present at t = 0: throughput without waiting for arrivals
            for r in reqs:
                r.arrival = 0.0
        return reqs

    eng = serving.ServingEngine(mu, max_concurrent=6)
    served_batch = eng.serve(stream()).summary()
    served_batch_burst = eng.serve(stream(burst=True)).summary()
    eng.close()
    # lane-level admission: propagation requests enter device-resident slot
    # pools as slots free up (the native server), corrections in merged batches
    eng = serving.ServingEngine(mu, max_concurrent=6, slots=True)
    eng.serve(serving.poisson_requests(200.0, 0.05, mu, seed=2, manifold_seeds=seeds, size_scale=0.05))  # warm
    served = eng.serve(stream()).summary()
    served_burst = eng.serve(stream(burst=True)).summary()
    eng.close()
    seq = serving.run_sequential(stream(), mu).summary()
    seq_burst = serving.run_sequential(stream(burst=True), mu).summary()
    out = {"workload": "serving mix, Poisson 200 req/s x 1 s (manifold / correct / synodic)", "metric": METRIC,
           "value": served_burst["traj_steps_per_s"], "unit": UNIT, "ms": served_burst["wall_s"] * 1e3,
           "config": {"rate_hz": 200, "window_s": 1.0},
           "p50_ms": served["p50_ms"], "p99_ms": served["p99_ms"],
           "timing": "host wall clock of the served stream (arrival to completion per request for p50/p99)",
           "form": "slot-level continuous batching (native server pools for manifold / synodic, merged "
                   "correction batches)",
           "served_poisson": served, "sequential_plain_poisson": seq, "served_burst": served_burst,
           "sequential_plain_burst": seq_burst,
           "merged_batches_poisson": served_batch, "merged_batches_burst": served_batch_burst,
           "speedup_vs_plain": served_burst["traj_steps_per_s"] / seq_burst["traj_steps_per_s"],
           "roofline": {"bound": "fp64", "note": "the served batches run the manifold, section and correction kernels; see their "
                                                  "roofline entries"}}
    if cpu:
        from oracle import hgo
        hgo.set_mode(hgo.MODE_NUMBA)
        th = os.cpu_count() or 1
        reqs = stream()
        rng = np.random.default_rng(7)
        man = np.concatenate([r.payload for r in reqs if r.kind == "manifold"])
        syn = np.concatenate([r.payload for r in reqs if r.kind == "synodic"])
        man = man[rng.choice(len(man), min(len(man), 256), replace=False)]
        syn = syn[rng.choice(len(syn), min(len(syn), 256), replace=False)]

        def one():
            a = hgo.dop853_event_batch(man, 0.0, TF, mu, 0, 1 - mu, 0, 1, max_step=1e4, fwd=-1, flip=(0, 6),
                                       threads=th)
            b = hgo.dop853_event_batch(syn, 0.0, 20.0, mu, 1, 0.0, -1, 8, rtol=1e-11, atol=1e-11, max_step=1e4,
                                       threads=th)
            return int(a["n_accept"].sum() + b["n_accept"].sum())
        v, dt, n = _cpu_loop(one, 2.0)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": th, "kind": "port",
                               "sample": f"256 manifold seeds + 256 synodic states drawn from the stream's requests, "
                                         f"repeated: {n} accepted steps in {dt:.1f} s (CPU oracle, numba lowering; "
                                         f"the CPU path has no serving form, so this is its propagation rate on "
                                         f"the mix's trajectories)"}
    return out


def bench_serving(args):
    import torch
    dev = torch.device("cuda", 0)
    _print_secondary(sec_serving(args.steps, dev, _peak(dev), cpu=not args.no_cpu_baseline))


def bench_continuation(args):
    """Halo-family continuation: 64 families (corrected L1/L2 halos, Az 0.05-0.3) continued in z for 12
    members each with the secant stepper; every round corrects the next member of all families in one
    batched correction."""
    import torch
    from hiten_gb300 import continuation as Cn
    from hiten_gb300 import corrector, halo
    from hiten_gb300 import workloads as W
    mu = W.MU_EM
    rng = np.random.default_rng(3)
    pts = np.repeat([1, 2], 32)
    az = rng.uniform(0.05, 0.3, 64)
    g = np.concatenate([halo.third_order_guess(mu, 1, az[:32], "southern"),
                        halo.third_order_guess(mu, 2, az[32:], "southern")])
    seed = corrector.correct_halo(g, mu)
    ok = seed.status == 0
    opts = Cn.ContinuationOptions(step=(0.002,), max_members=12)
    Cn.continue_halo_families(seed.x0[ok][:4], seed.period[ok][:4], mu, options=opts)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = Cn.continue_halo_families(seed.x0[ok], seed.period[ok], mu, options=opts)
    torch.cuda.synchronize()
    s = time.perf_counter() - t0
    members = sum(r.accepted_count - 1 for r in res)
    _line("halo-family continuation, 64 families x 12 members (secant, z)", "family members/s", members / s,
          "members/s", s * 1e3, {"families": int(ok.sum()), "members": 12,
                                 "l1_families": int(np.sum(pts[ok] == 1)), "l2_families": int(np.sum(pts[ok] == 2))},
          accepted=members, rejected=sum(r.rejected_count for r in res),
          rounds=max(r.iterations for r in res))


def bench_connections(args):
    """Connections between two synthetic sections of 65536 points each (noisy closed curves on the
    (y, vy) plane, as manifold cuts look), eps = 1e-4: the radius pairing in both directions and the
    nearest neighbours of both sets (4 all-pairs searches of 4.3e9 pairs), then the host refinement."""
    import torch
    from hiten_gb300.connections import find_connections
    n = 65536
    rng = np.random.default_rng(5)

    def curve(ph):
        s = rng.uniform(0, 1, n)
        return np.c_[0.1 * np.cos(2 * np.pi * s + ph) + rng.normal(0, 1e-4, n),
                     0.3 * np.sin(2 * np.pi * s + ph) + rng.normal(0, 1e-4, n)]

    pu, ps = curve(0.0), curve(0.3)
    Xu = np.c_[np.full(n, 0.85), pu[:, 0], np.zeros(n), rng.normal(0, 1e-3, n), pu[:, 1], rng.normal(0, 1e-3, n)]
    Xs = np.c_[np.full(n, 0.85), ps[:, 0], np.zeros(n), rng.normal(0, 1e-3, n), ps[:, 1], rng.normal(0, 1e-3, n)]
    run = lambda: find_connections(pu, ps, Xu, Xs, eps=1e-4, dv_tol=1e-2, bal_tol=1e-4)
    run()
    torch.cuda.synchronize()
    ts = []
    for _ in range(max(2, args.steps // 4)):
        t0 = time.perf_counter()
        res, meta = run()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    sec = statistics.median(ts)
    # the four all-pairs searches alone (device arrays resident, CUDA events)
    from hiten_gb300.connections import GpuSectionMatcher
    m = GpuSectionMatcher()
    R = float(max(np.abs(pu).max(), np.abs(ps).max()))
    qu, qs = torch.as_tensor(pu, device="cuda"), torch.as_tensor(ps, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    search = []
    for _ in range(3):
        ev[0].record()
        m.radius_best(qu, qs, 1e-4, R)
        m.radius_best(qs, qu, 1e-4, R)
        m.nearest(qu, R)
        m.nearest(qs, R)
        ev[1].record()
        torch.cuda.synchronize()
        search.append(ev[0].elapsed_time(ev[1]))
    pair_tests = 4.0 * n * n
    _line("connections, 65536 x 65536 section points, eps 1e-4", "pair tests/s", pair_tests / sec, "pairs/s",
          sec * 1e3, {"points_u": n, "points_s": n, "eps": 1e-4}, connections=len(res),
          pairs_considered=meta.get("pairs_considered", 0), gpu_search_ms=statistics.median(search))


EXTRA = {"fixed_stm": bench_fixed_stm, "section": bench_section, "synodic_detect": bench_synodic_detect,
         "correct": bench_correct,
         "serving": bench_serving, "continuation": bench_continuation, "connections": bench_connections}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the other workloads (RK8 + STM, section, correction, serving) measured after the headline")
    ap.add_argument("--plan", default=None,
                    help="force an execution plan by name (autotune.plan_name), e.g. scheduled_seg16")
    ap.add_argument("--workload", default="manifold", choices=["manifold"] + sorted(EXTRA),
                    help="manifold (the headline); the others print one secondary line each")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload != "manifold":
        return EXTRA[args.workload](args)

    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    from hiten_gb300 import _lib
    from hiten_gb300 import autotune
    from hiten_gb300 import manifold as M
    from hiten_gb300 import propagate as P
    from hiten_gb300 import workloads as W
    mu = W.MU_EM

    seeds = make_seeds(dev)
    N = len(seeds)
    seeds_dev = torch.as_tensor(seeds, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > L2
    stream = torch.cuda.current_stream(dev)

    def run(scheduled):
        return M.propagate_to_plane(seeds_dev, mu, tf=TF, forward=-1, device=dev, scheduled=scheduled)

    for _ in range(max(args.warmup, 3)):
        r = run(False)
    torch.cuda.synchronize(dev)
    # execution plan (single-pass launch shape or host-scheduled segments)
    # chosen by measurement on this workload; results are identical for all
    plans = autotune.DOP853_PLANS
    if args.plan:
        plans = [p for p in plans if autotune.plan_name(p) == args.plan]
        if not plans:
            raise SystemExit(f"unknown plan {args.plan}")
    plan, plan_ms = autotune.tune_dop853(f"manifold_{N}", run, plans=plans, device=dev)
    sched = plan["scheduled"]

    # the timed steps: the same call prepared once (propagate.Dop853Batch: inputs copied into static
    # device buffers, outputs and workspace allocated once), the bits of run(sched) -- checked here
    batch = P.Dop853Batch(N, 6, 0.0, TF, mu, rtol=1e-12, atol=1e-12, max_step=1e4, fwd=-1, flip=(0, 6),
                          event=P.EventSpec(index=0, offset=1.0 - mu, direction=0, max_hits=1), scheduled=sched,
                          device=dev)

    def one_step():
        return batch.run(seeds_dev)

    # plain form: one kernel call per trajectory, the reference's call
    # granularity (one _propagate_dynsys per seed), on a bounded sample
    n_plain = 64
    torch.cuda.synchronize(dev)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    plain_res = [M.propagate_to_plane(seeds_dev[i:i + 1], mu, tf=TF, forward=-1, device=dev) for i in range(n_plain)]
    p1.record(stream)
    torch.cuda.synchronize(dev)
    plain_acc = sum(int(x.n_accept.sum().item()) for x in plain_res)
    plain_value = plain_acc / (p0.elapsed_time(p1) * 1e-3)

    # the clock sampler starts here, ahead of the warm-up steps, so that its start-up is over before
    # the timed region; it is stopped after the timed steps, on every path
    clk = ClockSampler(local).__enter__()
    try:
        for _ in range(max(args.warmup, 3)):
            one_step()
        torch.cuda.synchronize(dev)
        _ref = run(sched)
        _got = one_step()
        if not (torch.equal(_ref.y_end, _got.y_end) and torch.equal(_ref.n_accept, _got.n_accept)
                and torch.equal(_ref.hit_t.nan_to_num(), _got.hit_t.nan_to_num())):
            raise SystemExit("prepared batch and propagate_dop853 disagree")

        # ---- device-resident timing (CUDA events on the launching stream)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        H = _lib.handle(local)
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)
        launches0 = H.kernel_launches()
        gc.collect()
        gc.disable()  # no collector pause inside the host-synchronised steps
        try:
            clk.begin()
            results = []
            for i in range(args.steps):
                flush.fill_(float(i))
                evs[i][0].record(stream)
                r = one_step()
                evs[i][1].record(stream)
                results.append(r)
            torch.cuda.synchronize(dev)
            clk.end()
        finally:
            gc.enable()
    finally:
        clk.__exit__(None, None, None)
    launches = H.kernel_launches() - launches0
    if world > 1:
        dist.barrier()
    clocks = clk.summary()
    times_ms = [a.elapsed_time(b) for a, b in evs]
    # every step propagates the same seeds into the batch's buffers (the same bits each time), so the
    # last step's counts are every step's
    r = results[-1]
    acc = len(results) * int(r.n_accept.sum().item())
    att = len(results) * int(r.n_accept.sum().item() + r.n_reject.sum().item())
    value, total_s = whole_job_rate(acc, sum(times_ms) * 1e-3, device=dev)
    total_ms = total_s * 1e3
    att_rate, _ = whole_job_rate(att, sum(times_ms) * 1e-3, device=dev)
    kernel_ms = total_ms / args.steps
    flops = FLOPS_PER_ATTEMPT_D6 * att / args.steps
    peak = P.fp64_peak_tflops(dev)

    # ---- end to end through the public API (pinned host seeds, H2D + D2H inside)
    host_seeds = torch.as_tensor(seeds).pin_memory()
    h2d = host_seeds.numel() * 8

    # the drop-in's results (separate tensors) are read back into pinned host buffers allocated once
    # (no host allocation or page faults inside the timed steps); one synchronisation per step
    out_host = {}

    def fetch(r):
        parts = (("y_end", r.y_end), ("hit_y", r.hit_y), ("hit_t", r.hit_t), ("n_acc", r.n_accept))
        for name, t in parts:
            buf = out_host.get(name)
            if buf is None or buf.shape != t.shape or buf.dtype != t.dtype:
                buf = out_host[name] = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
            buf.copy_(t, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()
        n_acc = out_host["n_acc"]
        return int(n_acc.sum()), sum(out_host[k].numel() * out_host[k].element_size() for k, _ in parts)

    def e2e_step():  # the prepared call (the timed steps' API) from pinned host memory; every output of the
        # batch read back in one copy of its output arena (to_host)
        batch.run(host_seeds)
        h = batch.to_host()
        return int(h.n_accept.sum()), batch.out.numel()

    def e2e_dropin_step():  # the reference-shaped per-call API
        return fetch(M.propagate_to_plane(host_seeds, mu, tf=TF, forward=-1, device=dev, scheduled=sched))

    def e2e_rate(step):
        for _ in range(max(args.warmup, 3)):  # untimed, like the device-resident steps
            step()
        acc_, d2h_ = 0, 0
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)
        gc.collect()
        gc.disable()
        try:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                n, d2h_ = step()
                acc_ += n
            torch.cuda.synchronize(dev)
            dt = time.perf_counter() - t0
        finally:
            gc.enable()
        return whole_job_rate(acc_, dt, device=dev)[0], d2h_

    e2e_value, d2h = e2e_rate(e2e_step)
    e2e_dropin_value, _ = e2e_rate(e2e_dropin_step)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = len(seeds)
        v, dt, n = cpu_reference(seeds, sample, threads, min_seconds=5.0)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"all {sample} seeds, repeated: {n} accepted steps in {dt:.1f} s, CPU oracle in "
                         f"numba-lowering mode, one trajectory per thread task"}

    def run_segment(g, seg):
        with P.tuning(device=dev, lanes_d6=g):
            return M.propagate_to_plane(seeds_dev, mu, tf=TF, forward=-1, device=dev, scheduled=False,
                                        segmented=True, seg_steps=seg, max_segments=1, finish=False)

    dom = dominant_launch(run_segment, plan, N, torch.cuda.get_device_properties(dev).multi_processor_count,
                          stream)

    # the other workloads of the metric, each measured in this run after the headline
    # (rank 0 of a single-GPU run; replicas add nothing to them)
    secondary = None
    if rank == 0 and world == 1 and not args.no_secondary:
        cpu_ok = not args.no_cpu_baseline
        secondary = {}
        for key, fn in (("fixed_rk8_stm_1024x3000", lambda: sec_fixed_stm(args.steps, dev, peak, cpu_ok)),
                        ("section_65536", lambda: sec_section(args.steps, dev, peak, cpu_ok)),
                        ("halo_correction_2048", lambda: sec_correct(args.steps, dev, peak, cpu_ok)),
                        ("serving_poisson_200hz", lambda: sec_serving(args.steps, dev, peak, cpu_ok, seeds=seeds))):
            t0 = time.perf_counter()
            try:
                secondary[key] = fn()
            except Exception as e:  # a failing secondary must not hide the headline
                secondary[key] = {"error": f"{type(e).__name__}: {e}"}
            secondary[key]["wall_s"] = time.perf_counter() - t0

    if rank == 0:
        prof = os.path.join(HERE, "profiles", "traffic_dop853_manifold.json")
        traffic, pipe = None, None
        if os.path.exists(prof):
            with open(prof) as f:
                rec = json.load(f)
            traffic = rec.get("dram_bytes_per_launch")
            pipe = {k: rec[k] for k in ("fp64_pipe_active", "fp64_issue_frac", "threads_per_instruction") if k in rec}
            pipe["source"] = ("from profiles/traffic_dop853_manifold.json (ncu of the dominant launch, "
                              "profiles/dop853_manifold_16384.md), not measured in this run")
        step_achieved = flops / (kernel_ms * 1e-3) / 1e12
        if dom is not None:
            g, dom_ms, dom_att = dom
            achieved = FLOPS_PER_ATTEMPT_D6 * dom_att / (dom_ms * 1e-3) / 1e12
            dom_info = {"kernel": f"dop853_kernel<{g}, false> (first scheduled segment: {N} live trajectories, "
                                  f"{int(plan.get('seg_steps', 16))} attempted steps each at most)",
                        "ms": dom_ms, "attempted_steps": dom_att,
                        "timing": "CUDA events on the launching stream around one segmented call issued "
                                  "behind a device sleep (its set-up and crossing refinement included), "
                                  "median of 3"}
        else:
            achieved, dom_info = step_achieved, {"kernel": "the single-pass launch", "ms": kernel_ms}
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config(world),
               "step_ms": {"min": min(times_ms), "median": statistics.median(times_ms), "max": max(times_ms)},
               "attempted_steps_per_s": att_rate,
               "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                            "frac": achieved / peak if peak else None, "traffic": traffic,
                            "traffic_scope": "DRAM bytes of one launch of the dominant kernel (the timed launch "
                                             "above, captured by ncu through its NVTX range); from "
                                             "profiles/traffic_dop853_manifold.json, not measured in this run",
                            "peak_source": "measured: DFMA throughput probe (hg_probe_fp64_peak) on this GPU; "
                                           "MEASURED_PEAKS.json has no FP64 entry",
                            "flops_per_attempted_step": FLOPS_PER_ATTEMPT_D6,
                            "dominant_launch": dom_info, "step_achieved": step_achieved,
                            "fp64_pipe": pipe},
               "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "api": "propagate.Dop853Batch.run from pinned host seeds (the timed steps' prepared call), "
                              "every output read back by Dop853Batch.to_host in one copy",
                       "dropin": {"value": e2e_dropin_value, "unit": UNIT,
                                  "api": "manifold.propagate_to_plane from pinned host seeds (per-call setup)"}},
               "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": launches,
               "plan": {"chosen": autotune.plan_name(plan), "autotune_ms": plan_ms},
               "plain_gpu": {"value": plain_value, "unit": UNIT,
                             "form": f"one kernel call per trajectory (reference call granularity), "
                                     f"{n_plain}-trajectory sample"},
               "library": os.path.basename(_lib.load()._name)}
        if secondary is not None:
            out["secondary"] = secondary
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
