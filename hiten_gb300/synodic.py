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
"""
import ctypes as C

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
