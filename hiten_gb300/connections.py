"""Heteroclinic / impulsive connections between two synodic sections.

Mirrors connections/backends.py:410-540 (``_ConnectionsBackend.run``): pair
the unstable-side section points with the stable-side ones within ``eps``,
keep mutual nearest pairs, refine each on the segments to the points' own
nearest neighbours (the closest points of two 2-D segments), interpolate
the states there and classify the velocity jump.  The two all-pairs searches
(radius pairing with each point's nearest partner, nearest neighbours within
a set) and the per-pair segment refinement run on the GPU (``hg_radius_best``,
``hg_nearest_neighbor``, ``hg_connection_refine``); the velocity jumps (numpy's
norm, whose BLAS dot order is the host's) and the result records are made on
the host.  A matcher without ``refine`` (the CPU oracle's, in the tests) takes
the same arithmetic in numpy.
"""
import ctypes as C
import gc
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from . import propagate as P


@dataclass(slots=True)
class ConnectionResult:
    """connections/types.py:60-120 (_ConnectionResult)."""

    kind: str
    delta_v: float
    point2d: tuple
    state_u: np.ndarray
    state_s: np.ndarray
    index_u: int
    index_s: int
    trajectory_index_u: int
    trajectory_index_s: int


class GpuSectionMatcher:
    """The two all-pairs searches and the segment refinement on the GPU."""

    def __init__(self, device=None):
        self.device = P._device(device)

    def _xy(self, pts):
        if isinstance(pts, torch.Tensor):  # (n, 2) already on a device
            t = pts.to(device=self.device, dtype=torch.float64)
        else:
            t = torch.as_tensor(np.ascontiguousarray(pts, dtype=np.float64), device=self.device)
        return t[:, 0].contiguous(), t[:, 1].contiguous()

    def _workspace(self, L, n):
        """The FP32 point copy's workspace for n points (grown, then reused)."""
        need = int(L.hg_points_workspace_bytes(int(n)))
        ws = getattr(self, "_ws", None)
        if ws is None or ws.numel() < max(need, 256):
            ws = torch.empty(max(need, 256), dtype=torch.uint8, device=self.device)
            self._ws = ws
        return ws, ws.numel()

    def radius_best(self, q, r, eps, coord_max):
        L = _lib.load()
        nq, nr = q.shape[0], r.shape[0]
        qx, qy = self._xy(q)
        rx, ry = self._xy(r)
        cnt = torch.empty(nq, dtype=torch.int32, device=self.device)
        bi = torch.empty(nq, dtype=torch.int32, device=self.device)
        bd = torch.empty(nq, dtype=torch.float64, device=self.device)
        st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        ws, wsb = self._workspace(L, nr)
        with torch.cuda.device(self.device):
            rc = L.hg_radius_best(nq, P._ptr(qx), P._ptr(qy), nr, P._ptr(rx), P._ptr(ry), float(eps), float(coord_max),
                                  P._ptr(cnt), P._ptr(bi), P._ptr(bd), P._ptr(ws), wsb, st)
        if rc != _lib.HG_OK:
            raise _lib.HitenGpuError(rc, "hg_radius_best failed")
        return cnt.cpu().numpy().astype(np.int64), bi.cpu().numpy().astype(np.int64), bd.cpu().numpy()

    def nearest(self, p, coord_max):
        L = _lib.load()
        n = p.shape[0]
        x, y = self._xy(p)
        out = torch.empty(n, dtype=torch.int32, device=self.device)
        st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        ws, wsb = self._workspace(L, n)
        with torch.cuda.device(self.device):
            rc = L.hg_nearest_neighbor(n, P._ptr(x), P._ptr(y), float(coord_max), P._ptr(out), P._ptr(ws), wsb, st)
        if rc != _lib.HG_OK:
            raise _lib.HitenGpuError(rc, "hg_nearest_neighbor failed")
        return out.cpu().numpy().astype(np.int64)


    def refine(self, pu, ps, Xu, Xs, I, IU, J, JS, ok):
        """Closest points, interpolated states and midpoints of the pairs
        (``hg_connection_refine``): (xu (n, 6), xs (n, 6), ptx, pty) on the host."""
        L = _lib.load()
        n = int(I.shape[0])
        dev = self.device

        def up(a, dt):
            return torch.as_tensor(np.ascontiguousarray(a, dtype=dt), device=dev)

        ti, tiu, tj, tjs = (up(a, np.int32) for a in (I, IU, J, JS))
        tok = up(ok, np.uint8)
        tpu, tps, tXu, tXs = (up(a, np.float64) for a in (pu, ps, Xu, Xs))
        xu = torch.empty((max(n, 1), 6), dtype=torch.float64, device=dev)
        xs = torch.empty_like(xu)
        pt = torch.empty((max(n, 1), 2), dtype=torch.float64, device=dev)
        st = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        with torch.cuda.device(dev):
            rc = L.hg_connection_refine(n, P._ptr(ti), P._ptr(tiu), P._ptr(tj), P._ptr(tjs), P._ptr(tok),
                                        int(pu.shape[0]), P._ptr(tpu), P._ptr(tXu), int(ps.shape[0]), P._ptr(tps),
                                        P._ptr(tXs), P._ptr(xu), P._ptr(xs), P._ptr(pt), st)
        if rc != _lib.HG_OK:
            raise _lib.HitenGpuError(rc, "hg_connection_refine failed")
        pt = pt[:n].cpu().numpy()
        return xu[:n].cpu().numpy(), xs[:n].cpu().numpy(), pt[:, 0].copy(), pt[:, 1].copy()


def closest_points_on_segments_2d(a0x, a0y, a1x, a1y, b0x, b0y, b1x, b1y):
    """connections/backends.py:237-320, the same scalar operations."""
    ux = a1x - a0x
    uy = a1y - a0y
    vx = b1x - b0x
    vy = b1y - b0y
    wx = a0x - b0x
    wy = a0y - b0y
    A = ux * ux + uy * uy
    B = ux * vx + uy * vy
    Cc = vx * vx + vy * vy
    D = ux * wx + uy * wy
    E = vx * wx + vy * wy
    den = A * Cc - B * B
    s = 0.0
    t = 0.0
    if den > 0.0:
        s = (B * E - Cc * D) / den
        t = (A * E - B * D) / den
    if s < 0.0:
        s = 0.0
        if Cc > 0.0:
            t = E / Cc
    elif s > 1.0:
        s = 1.0
        if Cc > 0.0:
            t = (E + B) / Cc
    if t < 0.0:
        t = 0.0
        if A > 0.0:
            s = -D / A
            if s < 0.0:
                s = 0.0
            elif s > 1.0:
                s = 1.0
    elif t > 1.0:
        t = 1.0
        if A > 0.0:
            s = (B - D) / A
            if s < 0.0:
                s = 0.0
            elif s > 1.0:
                s = 1.0
    return s, t, a0x + s * ux, a0y + s * uy, b0x + t * vx, b0y + t * vy


def closest_points_on_segments_2d_batch(a0x, a0y, a1x, a1y, b0x, b0y, b1x, b1y):
    """closest_points_on_segments_2d for arrays: the same expressions and the
    same order of the clamping branches, elementwise."""
    ux = a1x - a0x
    uy = a1y - a0y
    vx = b1x - b0x
    vy = b1y - b0y
    wx = a0x - b0x
    wy = a0y - b0y
    A = ux * ux + uy * uy
    B = ux * vx + uy * vy
    Cc = vx * vx + vy * vy
    D = ux * wx + uy * wy
    E = vx * wx + vy * wy
    den = A * Cc - B * B
    with np.errstate(divide="ignore", invalid="ignore"):
        pos = den > 0.0
        s = np.where(pos, (B * E - Cc * D) / den, 0.0)
        t = np.where(pos, (A * E - B * D) / den, 0.0)
        lo, hi = s < 0.0, s > 1.0
        t = np.where(lo & (Cc > 0.0), E / Cc, t)
        t = np.where(~lo & hi & (Cc > 0.0), (E + B) / Cc, t)
        s = np.where(lo, 0.0, np.where(hi, 1.0, s))
        tlo, thi = t < 0.0, t > 1.0
        s_lo = np.clip(-D / A, 0.0, 1.0)
        s_hi = np.clip((B - D) / A, 0.0, 1.0)
        s = np.where(tlo & (A > 0.0), s_lo, s)
        s = np.where(~tlo & thi & (A > 0.0), s_hi, s)
        t = np.where(tlo, 0.0, np.where(thi, 1.0, t))
    return s, t, a0x + s * ux, a0y + s * uy, b0x + t * vx, b0y + t * vy


def velocity_jumps(dvv):
    """|dv| of each row of dvv (n, 3) as ``np.linalg.norm(dvv[k])`` computes
    it: the square root of the row's BLAS dot product with itself
    (``np.vecdot`` runs the same dot routine per row)."""
    dvv = np.ascontiguousarray(dvv, dtype=np.float64)
    if hasattr(np, "vecdot"):
        return np.sqrt(np.vecdot(dvv, dvv))
    return np.array([np.linalg.norm(r) for r in dvv], dtype=np.float64)


def find_connections(points_u, points_s, states_u, states_s, traj_indices_u=None, traj_indices_s=None, eps=1e-3,
                     dv_tol=1e-3, bal_tol=1e-6, max_seg_len=1e9, matcher=None, device=None):
    """Connections between the unstable-side section (points_u (N, 2),
    states_u (N, 6)) and the stable-side one (points_s, states_s).
    Returns (results sorted by delta_v, metadata)."""
    pu = np.ascontiguousarray(points_u, dtype=np.float64).reshape(-1, 2)
    ps = np.ascontiguousarray(points_s, dtype=np.float64).reshape(-1, 2)
    Xu = np.asarray(states_u, dtype=np.float64)
    Xs = np.asarray(states_s, dtype=np.float64)
    if pu.size == 0 or ps.size == 0:
        return [], {}
    m = matcher or GpuSectionMatcher(device)
    R = float(max(np.max(np.abs(pu)), np.max(np.abs(ps))))
    cnt_u, best_u, d2_u = m.radius_best(pu, ps, eps, R)
    total = int(cnt_u.sum())
    if total == 0:
        return [], {}
    _, best_s, d2_s = m.radius_best(ps, pu, eps, R)
    # mutual nearest pairs, in the order of the unstable-side index
    cand = np.nonzero(cnt_u > 0)[0]
    jb = best_u[cand]
    keep = (best_s[jb] == cand) & (d2_s[jb] == d2_u[cand])
    I, J = cand[keep], jb[keep]
    if I.size == 0:
        return [], {}
    nn_u = m.nearest(pu, R) if pu.shape[0] >= 2 else np.full(pu.shape[0], -1, dtype=np.int64)
    nn_s = m.nearest(ps, R) if ps.shape[0] >= 2 else np.full(ps.shape[0], -1, dtype=np.int64)
    iu, js = nn_u[I], nn_s[J]
    ok = ~((iu < 0) | (js < 0) | (iu == I) | (js == J))
    iu_c, js_c = np.where(ok, iu, I), np.where(ok, js, J)
    du = np.hypot(pu[iu_c, 0] - pu[I, 0], pu[iu_c, 1] - pu[I, 1])
    ds = np.hypot(ps[js_c, 0] - ps[J, 0], ps[js_c, 1] - ps[J, 1])
    ok &= ~((du > max_seg_len) | (ds > max_seg_len))
    if hasattr(m, "refine"):
        # on the device: the same scalar arithmetic per pair
        xu, xs, ptx, pty = m.refine(pu, ps, Xu, Xs, I, iu_c, J, js_c, ok)
    else:
        s, t, px, py, qx, qy = closest_points_on_segments_2d_batch(
            pu[I, 0], pu[I, 1], pu[iu_c, 0], pu[iu_c, 1], ps[J, 0], ps[J, 1], ps[js_c, 0], ps[js_c, 1])
        s = np.where(ok, s, 0.0)
        t = np.where(ok, t, 0.0)
        xu = np.where(ok[:, None], (1.0 - s)[:, None] * Xu[I] + s[:, None] * Xu[iu_c], Xu[I])
        xs = np.where(ok[:, None], (1.0 - t)[:, None] * Xs[J] + t[:, None] * Xs[js_c], Xs[J])
        ptx = np.where(ok, 0.5 * (px + qx), pu[I, 0])
        pty = np.where(ok, 0.5 * (py + qy), pu[I, 1])
    dvv = xu[:, 3:6] - xs[:, 3:6]
    dv = velocity_jumps(dvv)
    # accepted pairs in the order of a stable sort on delta_v (the reference
    # appends in candidate order and sorts the list by delta_v)
    sel = np.nonzero(dv <= dv_tol)[0]
    order = sel[np.argsort(dv[sel], kind="stable")]
    tu = np.asarray(traj_indices_u)[I[order]].astype(np.int64).tolist() if traj_indices_u is not None else [0] * order.size
    ts = np.asarray(traj_indices_s)[J[order]].astype(np.int64).tolist() if traj_indices_s is not None else [0] * order.size
    xu_o, xs_o = xu[order], xs[order]
    # positional fields (kind, delta_v, point2d, state_u, state_s, index_u, index_s, trajectory_index_u,
    # trajectory_index_s): several times cheaper than keywords at tens of thousands of results.  The
    # cyclic collector is paused while they are made (they hold no cycles): otherwise the allocations
    # trigger full collections that rescan every live result list, several times the build itself.
    gc_was_on = gc.isenabled()
    gc.disable()
    try:
        results = [ConnectionResult("ballistic" if d <= bal_tol else "impulsive", d, (x, y), su, ss, i, j, a, b)
                   for d, x, y, su, ss, i, j, a, b in zip(dv[order].tolist(), ptx[order].tolist(),
                                                           pty[order].tolist(), xu_o, xs_o, I[order].tolist(),
                                                           J[order].tolist(), tu, ts)]
    finally:
        if gc_was_on:
            gc.enable()
    return results, {"pairs_considered": total, "accepted": len(results)}
