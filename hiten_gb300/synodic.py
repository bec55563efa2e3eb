"""Synodic Poincare sections on the GPU.

Two forms, both with the reference's crossing semantics:

* `detect` -- the reference's SynodicMap path: crossings of an axis-aligned
  plane found on already-sampled trajectories (poincare/synodic/backend.py,
  `_detect_with_segment_refine` + `_order_and_dedup_hits`, defaults of
  types/services/maps.py:721-774: segment_refine = 50, tol_on_surface = 1e-6,
  dedup_time_tol = 1e-9, dedup_point_tol = 1e-6; the default map uses linear
  sub-segment interpolation because its `interp_kind` is a RefineConfig
  object, backend.py:762).  One GPU thread per trajectory.
* `integrate_and_detect` -- crossings refined on the DOP853 dense
  interpolant during integration (the kernel's multi-hit event), without
  storing samples at all.

`GpuSynodicDetectionBackend` is the plugin-level drop-in for the reference's
`_SynodicDetectionBackend` (same methods, request and response fields).
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import NamedTuple, Optional, Sequence

import numpy as np
import torch

from . import _lib
from . import propagate as P

AXES = {"x": 0, "y": 1, "z": 2, "vx": 3, "vy": 4, "vz": 5}


def _axis(a):
    return AXES[a.lower()] if isinstance(a, str) else int(a)


def detect(times, samples, section_axis="x", section_offset=0.0, plane_coords=("y", "vy"), direction=None,
           segment_refine=50, interp="linear", newton_max_iter=10, tol_on_surface=1e-6, dedup_time_tol=1e-9,
           dedup_point_tol=1e-6, max_hits=16, device=None):
    """Crossings on sampled trajectories.

    samples: (m, N, 6) (as `Dop853Result.samples`); times: (m,) shared or (m, N).
    Returns (hit_t (N, max_hits), hit_y (N, max_hits, 6), n_hits (N,)) on the device."""
    dev = P._device(device)
    S = torch.as_tensor(samples, dtype=torch.float64, device=dev)
    m, N, _ = S.shape
    soa = S.permute(0, 2, 1).contiguous()  # (m, 6, N)
    T = torch.as_tensor(np.asarray(times, dtype=np.float64) if not torch.is_tensor(times) else times,
                        dtype=torch.float64, device=dev)
    tld = 0 if T.ndim == 1 else N
    T = T.contiguous()
    ld = max(N, 1)
    hit_t = torch.full((max_hits, ld), float("nan"), dtype=torch.float64, device=dev)
    hit_y = torch.full((max_hits, 6, ld), float("nan"), dtype=torch.float64, device=dev)
    n_hits = torch.zeros(ld, dtype=torch.int32, device=dev)
    d = 0 if direction is None else int(direction)
    L = _lib.load()
    rc = L.hg_section_detect(N, m, C.c_void_p(soa.data_ptr()), ld, C.c_void_p(T.data_ptr()), tld,
                             _axis(section_axis), float(section_offset), d, _axis(plane_coords[0]),
                             _axis(plane_coords[1]), int(segment_refine), 1 if interp == "cubic" else 0,
                             int(newton_max_iter), float(tol_on_surface), float(dedup_time_tol),
                             float(dedup_point_tol), int(max_hits), C.c_void_p(hit_t.data_ptr()),
                             C.c_void_p(hit_y.data_ptr()), C.c_void_p(n_hits.data_ptr()), None,
                             C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if rc != _lib.HG_OK:
        raise _lib.HitenGpuError(rc, "hg_section_detect")
    return hit_t[:, :N].t(), hit_y[:, :, :N].permute(2, 0, 1), n_hits[:N]


def integrate_and_detect(states, mu, tf=20.0, section_axis="y", section_offset=0.0, direction=-1, max_hits=8,
                         rtol=1e-11, atol=1e-11, device=None):
    """DOP853 from every state to t = tf, recording up to max_hits crossings
    of the plane (refined on the dense interpolant as _dop853_refine_in_step)."""
    ev = P.EventSpec(index=_axis(section_axis), offset=float(section_offset),
                     direction=0 if direction is None else int(direction), max_hits=int(max_hits))
    return P.propagate_dop853(states, 0.0, float(tf), mu, rtol=rtol, atol=atol, max_step=1e4, event=ev,
                              device=device)


class SectionHit(NamedTuple):
    """One crossing, the fields of poincare/core/types.py:45-75 (_SectionHit)."""
    time: float
    state: np.ndarray
    point2d: np.ndarray
    trajectory_index: int


@dataclass
class SynodicRequest:
    """The fields of poincare/synodic/types.py:16-32 (SynodicBackendRequest)."""
    trajectories: Sequence
    normal: Sequence
    trajectory_indices: Sequence
    offset: float = 0.0
    plane_coords: tuple = ("y", "vy")
    interp_kind: str = "linear"
    segment_refine: int = 0
    tol_on_surface: float = 1e-12
    dedup_time_tol: float = 1e-9
    dedup_point_tol: float = 1e-12
    max_hits_per_traj: Optional[int] = None
    newton_max_iter: int = 4
    direction: Optional[int] = None
    metadata: dict = field(default_factory=dict)


@dataclass
class SynodicResponse:
    """The fields of poincare/synodic/types.py:35-60 (SynodicBackendResponse)."""
    hits: list
    points: np.ndarray
    states: np.ndarray
    times: Optional[np.ndarray]
    trajectory_indices: np.ndarray
    metadata: dict = field(default_factory=dict)


def _normal_axis(normal):
    n = np.asarray(normal, dtype=np.float64).ravel()
    nz = np.nonzero(n)[0]
    if n.size != 6 or nz.size != 1 or n[nz[0]] != 1.0:
        raise ValueError("the GPU section detection takes axis-aligned planes: the normal must be a unit "
                         "coordinate vector of the 6-dim synodic state")
    return int(nz[0])


class GpuSynodicDetectionBackend:
    """poincare/synodic/backend.py:662-887 (_SynodicDetectionBackend) on the
    GPU: the same methods (`detect_on_trajectory`, `run`), arguments and
    results (lists of SectionHit per trajectory in segment order, deduplicated;
    the flattened points / states / times / trajectory indices), computed by
    `hg_section_detect`, whose crossings are the oracle's bit for bit.

    The kernel implements the refined path the synodic map takes
    (segment_refine >= 1; the map's default is 50) for planes g = x_k - c
    (`normal` a unit coordinate vector, whose dot product with a state is x_k
    exactly).  Trajectories of unequal length are detected in one launch per
    distinct sample count (a padded sample would add an on-surface candidate
    the reference never forms); max_hits_per_traj = None is served by
    relaunching, with twice the cap, the trajectories that reached it (the
    kernel's scan stops at the cap)."""

    def __init__(self, device=None, initial_cap=32):
        self.device = device
        self.initial_cap = int(initial_cap)

    def detect_on_trajectory(self, times, states, *, normal, offset=0.0, plane_coords=("y", "vy"),
                             interp_kind="linear", segment_refine=0, tol_on_surface=1e-12, dedup_time_tol=1e-9,
                             dedup_point_tol=1e-12, max_hits_per_traj=None, newton_max_iter=4, direction=None,
                             trajectory_index=0):
        return self._detect([(times, states)], [trajectory_index], normal=normal, offset=offset,
                            plane_coords=plane_coords, interp_kind=interp_kind, segment_refine=segment_refine,
                            tol_on_surface=tol_on_surface, dedup_time_tol=dedup_time_tol,
                            dedup_point_tol=dedup_point_tol, max_hits_per_traj=max_hits_per_traj,
                            newton_max_iter=newton_max_iter, direction=direction)[0]

    def run(self, request):
        hits = self._detect(request.trajectories, request.trajectory_indices, normal=request.normal,
                            offset=request.offset, plane_coords=request.plane_coords,
                            interp_kind=request.interp_kind, segment_refine=request.segment_refine,
                            tol_on_surface=request.tol_on_surface, dedup_time_tol=request.dedup_time_tol,
                            dedup_point_tol=request.dedup_point_tol, max_hits_per_traj=request.max_hits_per_traj,
                            newton_max_iter=request.newton_max_iter, direction=request.direction)
        flat = [h for hs in hits for h in hs]
        return SynodicResponse(
            hits=hits,
            points=np.asarray([h.point2d for h in flat], dtype=float) if flat else np.empty((0, 2)),
            states=np.asarray([h.state for h in flat], dtype=float) if flat else np.empty((0, 6)),
            times=np.asarray([h.time for h in flat], dtype=float) if flat else None,
            trajectory_indices=(np.asarray([h.trajectory_index for h in flat], dtype=int) if flat
                                else np.empty((0,), dtype=int)),
            metadata={})

    def _detect(self, trajectories, indices, *, normal, offset, plane_coords, interp_kind, segment_refine,
                tol_on_surface, dedup_time_tol, dedup_point_tol, max_hits_per_traj, newton_max_iter, direction):
        if int(segment_refine) < 1:
            raise ValueError("the GPU section detection implements the refined path (segment_refine >= 1; the "
                             "synodic map's default is 50)")
        if interp_kind not in ("linear", "cubic"):
            raise ValueError(f"interp_kind must be 'linear' or 'cubic', not {interp_kind!r}")
        axis = _normal_axis(normal)
        pu, pv = (_axis(plane_coords[0]), _axis(plane_coords[1]))
        trajs = [(np.asarray(t, dtype=np.float64), np.asarray(s, dtype=np.float64)) for t, s in trajectories]
        idx = [int(i) for i in indices]
        if len(idx) != len(trajs):
            raise ValueError("one trajectory index per trajectory")
        out = [[] for _ in trajs]
        groups = {}
        for k, (t, s) in enumerate(trajs):
            if t.ndim != 1 or s.shape != (t.size, 6):
                raise ValueError("each trajectory is (times (n,), states (n, 6))")
            if t.size >= 2:
                groups.setdefault(t.size, []).append(k)
        for m, members in groups.items():
            # the reference appends a hit before testing the cap, so a cap of 0 keeps one hit
            cap = max(int(max_hits_per_traj), 1) if max_hits_per_traj is not None else self.initial_cap
            todo = members
            while todo:
                T = np.stack([trajs[k][0] for k in todo], axis=1)          # (m, n)
                S = np.stack([trajs[k][1] for k in todo], axis=1)          # (m, n, 6)
                ht, hy, nh, _ = _detect_raw(T, S, axis, offset, direction, (pu, pv), segment_refine,
                                             interp_kind == "cubic", newton_max_iter, tol_on_surface,
                                             dedup_time_tol, dedup_point_tol, cap, self.device)
                again = []
                for j, k in enumerate(todo):
                    # the scan stops at the cap: a trajectory that reached it may have more
                    if max_hits_per_traj is None and nh[j] >= cap:
                        again.append(k)
                        continue
                    out[k] = [SectionHit(time=float(ht[j, q]), state=hy[j, q].copy(),
                                         point2d=np.array([hy[j, q, pu], hy[j, q, pv]]), trajectory_index=idx[k])
                              for q in range(int(nh[j]))]
                cap *= 2
                todo = again
        return out


def _detect_raw(times, samples, axis, offset, direction, plane, segment_refine, cubic, newton_max_iter,
                tol_on_surface, dedup_time_tol, dedup_point_tol, max_hits, device):
    """hg_section_detect on (m, n) times and (m, n, 6) samples; host arrays
    hit_t (n, max_hits), hit_y (n, max_hits, 6), n_hits (n,), n_found (n,)."""
    dev = P._device(device)
    m, N, _ = samples.shape
    soa = torch.as_tensor(np.ascontiguousarray(samples.transpose(0, 2, 1)), device=dev)  # (m, 6, N)
    T = torch.as_tensor(np.ascontiguousarray(times), device=dev)                           # (m, N)
    hit_t = torch.full((max_hits, N), float("nan"), dtype=torch.float64, device=dev)
    hit_y = torch.full((max_hits, 6, N), float("nan"), dtype=torch.float64, device=dev)
    n_hits = torch.zeros(N, dtype=torch.int32, device=dev)
    n_found = torch.zeros(N, dtype=torch.int32, device=dev)
    d = 0 if direction is None else int(direction)
    L = _lib.load()
    rc = L.hg_section_detect(N, m, C.c_void_p(soa.data_ptr()), N, C.c_void_p(T.data_ptr()), N, int(axis),
                             float(offset), d, int(plane[0]), int(plane[1]), int(segment_refine), 1 if cubic else 0,
                             int(newton_max_iter), float(tol_on_surface), float(dedup_time_tol),
                             float(dedup_point_tol), int(max_hits), C.c_void_p(hit_t.data_ptr()),
                             C.c_void_p(hit_y.data_ptr()), C.c_void_p(n_hits.data_ptr()),
                             C.c_void_p(n_found.data_ptr()), C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if rc != _lib.HG_OK:
        raise _lib.HitenGpuError(rc, "hg_section_detect")
    return (hit_t.t().cpu().numpy(), hit_y.permute(2, 0, 1).cpu().numpy(), n_hits.cpu().numpy(),
            n_found.cpu().numpy())
