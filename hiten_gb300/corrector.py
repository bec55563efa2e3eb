"""Batched single-shooting Newton correction of halo orbits on the GPU.

Restates the reference's default halo correction (orbit.correct()):

* residual (corrector/operators.py:408-423): x_full = guess with the
  controls (x, vy) replaced; propagate to the first y = 0 crossing in the
  half-period window (poincare/singlehit/backend.py:164-280: DOP853
  rtol = atol = 1e-12, max_step = inf, over [0, pi - 1e-12], the returned
  time being 1e-12 + t_hit); r = (vx, vz) at the crossing;
* Jacobian (operators.py:437-450): Phi(t_event) from the 42-dim variational
  system (dynamics/rtbp.py:258-340: DOP853 1e-12, max_step 1e4, dense output
  at the final node), J = Phi[[3,5]][:, [0,4]] minus the halo quadratic term
  (types/services/orbits.py:917-948);
* Newton loop (corrector/backends/newton.py:100-143): stop when
  ||r||_inf < tol before the step; delta from np.linalg.solve (Tikhonov 1e-12
  when cond > 1e8, corrector/backends/base.py:187-245); Armijo backtracking
  (corrector/stepping/armijo.py:98-164: |delta|_inf capped at max_delta,
  alpha halved down to 1e-4, accept when |r(x+alpha d)| <= (1-0.1 alpha)|r|);
* period = 2 * event time of the corrected state (corrector/interfaces.py:48-74).

Every orbit of the batch iterates on its own schedule (uneven iteration
counts); each Newton sweep issues one batched event integration, one batched
STM integration and one batched event integration per Armijo level, over the
orbits still active.  The small 2x2 linear algebra runs in numpy exactly as
the reference does (stacked LAPACK calls give the same bits as single calls).
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from . import propagate as P
from .workloads import identity_stm_state

STATUS_OK = 0
STATUS_MAX_ITER = 4        # Newton did not converge in max_attempts
STATUS_NO_EVENT = 5        # no y = 0 crossing in the half-period window
STATUS_LINE_SEARCH = 6     # Armijo found no productive step


@dataclass
class HaloCorrectionOptions:
    """Defaults of _HaloOrbitCorrectionService (types/services/orbits.py:851-915)."""

    tol: float = 1e-12
    max_attempts: int = 50
    max_delta: float = 1e-2
    steps: int = 500
    alpha_reduction: float = 0.5
    min_alpha: float = 1e-4
    armijo_c: float = 0.1
    # Armijo trials evaluated per round and orbit (the next step fractions in
    # one propagation; results unchanged): None = as many as fill the
    # backend's latency-bound propagation size (1 for backends without one)
    trials_per_round: int = None
    cond_threshold: float = 1e8
    event_rtol: float = 1e-12
    event_atol: float = 1e-12
    stm_rtol: float = 1e-12
    stm_atol: float = 1e-12


class GpuShootingBackend:
    """The two propagations single shooting needs, batched on the GPU.

    ``spec_traj``: the event-leg size that still runs at the per-step latency
    floor (six lanes per trajectory, four warps per SM)."""

    def __init__(self, mu, options=None, device=None):
        self.mu = float(mu)
        self.o = options or HaloCorrectionOptions()
        self.device = device
        self.launches = 0
        self.attempts = {6: 0, 42: 0}  # attempted DOP853 steps of the event and STM legs
        import torch
        dev = P._device(device)
        self.spec_traj = 20 * torch.cuda.get_device_properties(dev).multi_processor_count

    def events(self, x_full):
        """First y = 0 crossing of every state: (t_event, x_event, found)."""
        ev = P.EventSpec(index=1, offset=0.0, direction=0, max_hits=1)
        span = max(0.0, np.pi - 1e-12)
        r = P.propagate_dop853(x_full, 0.0, span, self.mu, rtol=self.o.event_rtol, atol=self.o.event_atol,
                               max_step=np.inf, event=ev, device=self.device)
        self.launches += 1
        self.attempts[6] += int((r.n_accept + r.n_reject).sum())
        n = r.n_hits.cpu().numpy()
        t_rel = r.hit_t[:, 0].cpu().numpy()
        x_ev = r.hit_y[:, 0, :].cpu().numpy()
        found = (n > 0) & (t_rel < span) & (t_rel >= 0.0)
        return 1e-12 + t_rel, x_ev, found

    def stm(self, x_full, t_event):
        """Phi(t_event) of every state, (M, 6, 6)."""
        y0 = identity_stm_state(x_full)
        r = P.propagate_dop853(y0, 0.0, np.asarray(t_event, dtype=np.float64), self.mu, rtol=self.o.stm_rtol,
                               atol=self.o.stm_atol, max_step=1e4, flip=(36, 42), n_samples=int(self.o.steps),
                               sample_last_only=True, device=self.device)
        self.launches += 1
        self.attempts[42] += int((r.n_accept + r.n_reject).sum())
        return r.samples[0, :, :36].cpu().numpy().reshape(-1, 6, 6)


def _libm_pow(a, e):
    """Elementwise C `pow`: what the reference's numpy-scalar `**` computes
    (numpy's array `**` takes other paths: `x*x` for 2, SIMD kernels for
    fractional exponents, which differ in the last bit); one call into the
    library's host loop (`hg_host_pow`) instead of a Python call per element."""
    flat = np.ascontiguousarray(a, dtype=np.float64).ravel()
    out = np.empty_like(flat)
    if flat.size:
        _lib.load().hg_host_pow(flat.size, flat.ctypes.data_as(C.c_void_p), float(e), out.ctypes.data_as(C.c_void_p))
    return out.reshape(np.shape(a))


def halo_quadratic_term(x_ev, Phi, mu):
    """types/services/orbits.py:917-948 for a batch of orbits: the same
    expression tree as the reference's per-orbit numpy scalar code, with its
    powers through C `pow` and every +, -, *, / elementwise (identical to the
    scalar operations)."""
    x, y, z, vx, vy = (np.ascontiguousarray(x_ev[:, i]) for i in range(5))
    mu2 = 1 - mu
    y2 = _libm_pow(y, 2)
    z2 = _libm_pow(z, 2)
    rho_1 = 1 / _libm_pow((_libm_pow(x + mu, 2) + y2) + z2, 1.5)
    rho_2 = 1 / _libm_pow((_libm_pow(x - mu2, 2) + y2) + z2, 1.5)
    omega_x = (-((mu2 * (x + mu)) * rho_1) - ((mu * (x - mu2)) * rho_2)) + x
    DDx = 2 * vy + omega_x
    DDz = -((mu2 * z) * rho_1) - ((mu * z) * rho_2)
    small = np.abs(vy) < 1e-9
    vy = np.where(small, np.where(vy != 0, np.sign(vy) * 1e-9, 1e-9), vy)
    # [[DDx], [DDz]] @ Phi[[1], (0, 4)] / vy: a rank-one product, one multiply per entry
    p = Phi[:, 1, [0, 4]]
    out = np.empty((x_ev.shape[0], 2, 2))
    out[:, 0, :] = DDx[:, None] * p / vy[:, None]
    out[:, 1, :] = DDz[:, None] * p / vy[:, None]
    return out


def solve_delta(J, r, cond_threshold=1e8):
    """corrector/backends/base.py:187-245 for a stack of square systems."""
    cond = np.linalg.cond(J)
    reg = np.isnan(cond) | (cond > cond_threshold)
    Jr = J + reg[:, None, None] * (np.eye(J.shape[-1]) * 1e-12)
    Jr = np.where(reg[:, None, None], Jr, J)
    try:
        return np.linalg.solve(Jr, -r[..., None])[..., 0]
    except np.linalg.LinAlgError:
        out = np.empty_like(r)
        for i in range(J.shape[0]):
            try:
                out[i] = np.linalg.solve(Jr[i], -r[i])
            except np.linalg.LinAlgError:
                out[i] = np.linalg.lstsq(Jr[i], -r[i], rcond=None)[0]
        return out


@dataclass
class HaloCorrectionResult:
    x0: np.ndarray            # (N, 6) corrected initial states
    half_period: np.ndarray   # (N,)
    period: np.ndarray        # (N,)
    iterations: np.ndarray    # (N,)
    residual_norm: np.ndarray  # (N,)
    status: np.ndarray        # (N,)
    launches: int = 0


def correct_halo(guesses, mu, options=None, backend=None, device=None):
    """Correct a batch of halo guesses (N, 6); returns HaloCorrectionResult."""
    o = options or HaloCorrectionOptions()
    be = backend or GpuShootingBackend(mu, o, device=device)
    base = np.array(guesses, dtype=np.float64, copy=True)
    N = base.shape[0]
    ctrl = [0, 4]
    params = base[:, ctrl].copy()
    status = np.full(N, -1, dtype=np.int32)
    iters = np.zeros(N, dtype=np.int32)
    rnorm_out = np.full(N, np.nan)
    tev_out = np.full(N, np.nan)

    def full(p, rows):
        xf = base[rows].copy()
        xf[:, ctrl] = p
        return xf

    def residual(p, rows):
        t_ev, x_ev, found = be.events(full(p, rows))
        r = x_ev[:, [3, 5]] - np.zeros(2)
        norm = np.max(np.abs(r), axis=1)
        return r, norm, t_ev, x_ev, found

    active = np.arange(N)
    r, rn, tev, xev, found = residual(params[active], active)
    bad = ~found
    status[active[bad]] = STATUS_NO_EVENT
    keep = ~bad
    active, r, rn, tev, xev = active[keep], r[keep], rn[keep], tev[keep], xev[keep]

    for k in range(o.max_attempts):
        conv = rn < o.tol
        if conv.any():
            rows = active[conv]
            status[rows] = STATUS_OK
            iters[rows] = k
            rnorm_out[rows] = rn[conv]
            tev_out[rows] = tev[conv]
        keep = ~conv
        active, r, rn, tev, xev = active[keep], r[keep], rn[keep], tev[keep], xev[keep]
        if active.size == 0:
            break
        x_full = full(params[active], active)
        Phi = be.stm(x_full, tev)
        J = Phi[:, [3, 5], :][:, :, [0, 4]] - halo_quadratic_term(xev, Phi, mu)
        delta = solve_delta(J, r, o.cond_threshold)
        # Armijo line search, batched over the orbits still searching
        if o.max_delta is not None and not np.isinf(o.max_delta):
            dn = np.max(np.abs(delta), axis=1)
            cap = dn > o.max_delta
            delta[cap] = delta[cap] * (o.max_delta / dn[cap])[:, None]
        x0p = params[active].copy()
        alpha = np.ones(active.size)
        best = (x0p.copy(), rn.copy(), np.zeros(active.size), r.copy(), tev.copy(), xev.copy())
        new = [x0p.copy(), rn.copy(), r.copy(), tev.copy(), xev.copy()]
        pending = np.ones(active.size, dtype=bool)
        failed = np.zeros(active.size, dtype=bool)
        while pending.any():
            idx = np.nonzero(pending)[0]
            # the next S step fractions of every pending orbit in one
            # propagation (alpha, alpha r, ... by the same repeated products),
            # consumed below in the sequential order
            S = o.trials_per_round or max(1, min(8, getattr(be, "spec_traj", 1) // idx.size))
            A = np.empty((idx.size, S))
            a = alpha[idx].copy()
            for j in range(S):
                A[:, j] = a
                a = a * o.alpha_reduction
            trials = x0p[idx][:, None, :] + A[:, :, None] * delta[idx][:, None, :]
            rt, nt, tt, xt, ft = residual(trials.reshape(-1, 2), np.repeat(active[idx], S))
            rt, nt, tt, ft = rt.reshape(idx.size, S, 2), nt.reshape(idx.size, S), tt.reshape(idx.size, S), \
                ft.reshape(idx.size, S)
            xt = xt.reshape(idx.size, S, 6)
            deciding = np.ones(idx.size, dtype=bool)
            for j in range(S):
                u = np.nonzero(deciding)[0]
                if u.size == 0:
                    break
                q = idx[u]
                trial, nj, rj, tj, xj, fj = trials[u, j], nt[u, j], rt[u, j], tt[u, j], xt[u, j], ft[u, j]
                # an evaluation without a crossing is a failed residual: try a smaller step
                ok = fj & (nj <= (1.0 - o.armijo_c * alpha[q]) * rn[q])
                # accepted trials
                a_i = q[ok]
                for dst, src in zip(new, (trial, nj, rj, tj, xj)):
                    dst[a_i] = src[ok]
                pending[a_i] = False
                deciding[u[ok]] = False
                # rejected ones: remember the best finite trial, halve alpha
                rej = ~ok
                r_i = q[rej]
                better = fj[rej] & (nj[rej] < best[1][r_i])
                b_i = r_i[better]
                best[2][b_i] = alpha[b_i]
                for dst, src in zip((best[0], best[1], best[3], best[4], best[5]), (trial, nj, rj, tj, xj)):
                    dst[b_i] = src[rej][better]
                alpha[r_i] *= o.alpha_reduction
                stop = alpha[r_i] < o.min_alpha
                s_i = r_i[stop]
                pending[s_i] = False
                deciding[u[rej][stop]] = False
                g_i = s_i[best[2][s_i] > 0]
                for dst, src in zip(new, (best[0], best[1], best[3], best[4], best[5])):
                    dst[g_i] = src[g_i]
                failed[s_i[best[2][s_i] <= 0]] = True
        status[active[failed]] = STATUS_LINE_SEARCH
        iters[active[failed]] = k
        keep = ~failed
        params[active[keep]] = new[0][keep]
        active = active[keep]
        rn, r, tev, xev = new[1][keep], new[2][keep], new[3][keep], new[4][keep]
    else:
        # loop exhausted: final residual check (newton.py:130-143)
        if active.size:
            conv = rn < o.tol
            status[active[conv]] = STATUS_OK
            status[active[~conv]] = STATUS_MAX_ITER
            iters[active] = o.max_attempts
            rnorm_out[active] = rn
            tev_out[active] = tev
    x0 = base.copy()
    x0[:, ctrl] = params
    return HaloCorrectionResult(x0=x0, half_period=tev_out, period=2.0 * tev_out, iterations=iters,
                                residual_norm=rnorm_out, status=status, launches=getattr(be, "launches", 0))


def newton_step_norms(x0, mu, options=None, backend=None, device=None):
    """||dx||_inf of the Newton correction one more iteration would take at
    each state x0 (N, 6): the residual at the half-period crossing, the STM
    there and the step of the 2x2 solve (uncapped), as in correct_halo.  At a
    converged orbit this is the distance the iteration still sees to its
    fixed point; NaN where the crossing is not found."""
    o = options or HaloCorrectionOptions()
    be = backend or GpuShootingBackend(mu, o, device=device)
    x = np.atleast_2d(np.asarray(x0, dtype=np.float64))
    t_ev, x_ev, found = be.events(x)
    out = np.full(len(x), np.nan)
    if not found.any():
        return out
    xs, te, xe = x[found], t_ev[found], x_ev[found]
    r = xe[:, [3, 5]]
    Phi = be.stm(xs, te)
    J = Phi[:, [3, 5], :][:, :, [0, 4]] - halo_quadratic_term(xe, Phi, mu)
    out[found] = np.max(np.abs(solve_delta(J, r, o.cond_threshold)), axis=1)
    return out


def correct_halo_graph(guesses, mu, options=None, device=None, workspace=None):
    """correct_halo run on the device as one CUDA graph
    (``hg_correct_halo_graph``): every orbit's Newton iterations and Armijo
    line searches as nested conditional loops, no host round trip inside the
    correction.  ``workspace``: an optional uint8 device tensor of at least
    hg_correct_halo_graph_workspace_bytes(N) bytes (reused across calls so
    the cached graph stays valid; one is allocated when omitted).  Returns a
    HaloCorrectionResult."""
    import ctypes as C

    import torch

    from . import _lib
    o = options or HaloCorrectionOptions()
    dev = P._device(device)
    g = np.atleast_2d(np.asarray(guesses, dtype=np.float64))
    N = g.shape[0]
    L = _lib.load()
    need = int(L.hg_correct_halo_graph_workspace_bytes(max(N, 1)))
    if workspace is None or workspace.numel() < need + 256:
        workspace = torch.empty(need + 256, dtype=torch.uint8, device=dev)
    off = (-workspace.data_ptr()) % 256
    x = torch.as_tensor(g, device=dev).t().contiguous()
    half = torch.empty(max(N, 1), dtype=torch.float64, device=dev)
    resid = torch.empty(max(N, 1), dtype=torch.float64, device=dev)
    iters = torch.empty(max(N, 1), dtype=torch.int32, device=dev)
    status = torch.empty(max(N, 1), dtype=torch.int32, device=dev)
    no = _lib.hg_newton_opts(o.tol, o.max_attempts, np.inf if o.max_delta is None else o.max_delta,
                             o.alpha_reduction, o.min_alpha, o.armijo_c, o.cond_threshold, o.event_rtol,
                             o.event_atol, o.stm_rtol, o.stm_atol, o.steps)
    H = _lib.handle(dev.index or 0)
    with torch.cuda.device(dev):
        H.check(L.hg_correct_halo_graph(H.ptr, float(mu), N, P._ptr(x), max(N, 1), P._ptr(half), P._ptr(iters),
                                        P._ptr(resid), P._ptr(status), C.byref(no),
                                        C.c_void_p(workspace.data_ptr() + off), workspace.numel() - off,
                                        C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    st = status[:N].cpu().numpy().astype(np.int32)
    hp = half[:N].cpu().numpy()
    return HaloCorrectionResult(x0=x[:, :N].t().cpu().numpy(), half_period=hp, period=2.0 * hp,
                                iterations=iters[:N].cpu().numpy().astype(np.int64),
                                residual_norm=resid[:N].cpu().numpy(), status=st, launches=3)


def correct_halo_native(guesses, mu, options=None, device=None):
    """correct_halo through the library's native driver (``hg_correct_halo``):
    the same batched Newton/Armijo loop on the host side of the C ABI, for
    callers that bind the library without Python.  Returns a
    HaloCorrectionResult (launches not counted)."""
    import ctypes as C

    import torch

    from . import _lib
    o = options or HaloCorrectionOptions()
    dev = P._device(device)
    g = np.atleast_2d(np.asarray(guesses, dtype=np.float64))
    N = g.shape[0]
    x = torch.as_tensor(g, device=dev).t().contiguous()
    half = torch.empty(max(N, 1), dtype=torch.float64, device=dev)
    resid = torch.empty(max(N, 1), dtype=torch.float64, device=dev)
    iters = torch.empty(max(N, 1), dtype=torch.int32, device=dev)
    status = torch.empty(max(N, 1), dtype=torch.int32, device=dev)
    no = _lib.hg_newton_opts(o.tol, o.max_attempts, np.inf if o.max_delta is None else o.max_delta,
                             o.alpha_reduction, o.min_alpha, o.armijo_c, o.cond_threshold, o.event_rtol,
                             o.event_atol, o.stm_rtol, o.stm_atol, o.steps)
    H = _lib.handle(dev.index or 0)
    with torch.cuda.device(dev):
        H.check(H.lib.hg_correct_halo(H.ptr, float(mu), N, P._ptr(x), max(N, 1), P._ptr(half), P._ptr(iters),
                                      P._ptr(resid), P._ptr(status), C.byref(no),
                                      C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    st = status[:N].cpu().numpy().astype(np.int32)
    # the library's status codes are the corrector's: OK 0, max iterations 4,
    # no crossing 5, line search 6
    hp = half[:N].cpu().numpy()
    return HaloCorrectionResult(x0=x[:, :N].t().cpu().numpy(), half_period=hp, period=2.0 * hp,
                                iterations=iters[:N].cpu().numpy().astype(np.int64),
                                residual_norm=resid[:N].cpu().numpy(), status=st, launches=0)
