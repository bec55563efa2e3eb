"""ctypes front end of the CPU oracle (``oracle/hgo.c``).

Test infrastructure: imported by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` only, as the checker.  Each function
restates a reference routine (see ``hgo.h`` for the file:line map) and takes
plain numpy arrays.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

MODE_PYTHON = 0
MODE_NUMBA = 1
MODE_DEVICE = 2

_lib = None
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_LP = C.POINTER(C.c_long)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.hgo_set_mode.argtypes = [C.c_int]
        L.hgo_get_mode.restype = C.c_int
        L.hgo_fpow.argtypes = [C.c_double, C.c_double]
        L.hgo_fpow.restype = C.c_double
        L.hgo_rhs6.argtypes = [_DP, C.c_double, _DP]
        L.hgo_rhs42.argtypes = [_DP, C.c_double, _DP]
        L.hgo_fixed_rk.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                   _DP, _DP, C.c_int, _DP]
        L.hgo_fixed_rk.restype = C.c_int
        L.hgo_dop853_dense.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _DP, _DP,
                                       C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_long, _DP, _LP, _LP]
        L.hgo_dop853_dense.restype = C.c_int
        L.hgo_dop853_event.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _DP,
                                       C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_long, C.c_int, C.c_double, C.c_int, C.c_int,
                                       C.c_double, C.c_double, _DP, _DP, _IP, _DP, _DP, _LP, _LP]
        L.hgo_dop853_event.restype = C.c_int
        L.hgo_fixed_rk_batch.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                         C.c_int, _DP, _DP, C.c_int, C.c_int, _DP, C.c_int]
        L.hgo_fixed_rk_batch.restype = C.c_int
        L.hgo_dop853_event_batch.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                             _DP, C.c_double, C.c_double, C.c_double, C.c_double,
                                             C.c_double, C.c_double, C.c_long, C.c_int, C.c_double,
                                             C.c_int, C.c_int, C.c_double, C.c_double, _DP, _DP, _IP,
                                             _DP, _DP, _LP, _LP, _IP, C.c_int]
        L.hgo_dop853_event_batch.restype = C.c_int
        _lib = L
    return _lib


def _p(a, t=_DP):
    return a.ctypes.data_as(t)


class mode:
    """Context manager selecting how powers are evaluated (see hgo.h)."""

    def __init__(self, m):
        self.m = m

    def __enter__(self):
        self.old = lib().hgo_get_mode()
        lib().hgo_set_mode(self.m)
        return self

    def __exit__(self, *exc):
        lib().hgo_set_mode(self.old)


def set_mode(m):
    lib().hgo_set_mode(int(m))


def fpow(x, y):
    return lib().hgo_fpow(float(x), float(y))


def _flip(dim, fwd, flip):
    if flip is None:
        return 0, dim
    return int(flip[0]), int(flip[1])


def rhs(y, mu):
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.empty_like(y)
    (lib().hgo_rhs6 if y.size == 6 else lib().hgo_rhs42)(_p(y), float(mu), _p(out))
    return out


def fixed_rk(order, y0, t_vals, mu, fwd=1, flip=None):
    """integrators/rk.py:531-588 on one trajectory; returns (n, dim) states."""
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    t_vals = np.ascontiguousarray(t_vals, dtype=np.float64)
    dim = y0.size
    lo, hi = _flip(dim, fwd, flip)
    out = np.empty((t_vals.size, dim))
    st = lib().hgo_fixed_rk(int(order), dim, float(mu), int(fwd), lo, hi, _p(y0), _p(t_vals),
                            t_vals.size, _p(out))
    return out, st


def fixed_rk_batch(order, y0, t_vals, mu, out_every=1, fwd=1, flip=None, threads=None):
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    t_vals = np.ascontiguousarray(t_vals, dtype=np.float64)
    N, dim = y0.shape
    lo, hi = _flip(dim, fwd, flip)
    n_out = (t_vals.size - 1) // out_every + 1
    out = np.empty((N, n_out, dim))
    th = threads or os.cpu_count() or 1
    st = lib().hgo_fixed_rk_batch(int(order), dim, float(mu), int(fwd), lo, hi, N, _p(y0), _p(t_vals),
                                  t_vals.size, int(out_every), _p(out), int(th))
    return out, st


def dop853_dense(y0, t_eval, mu, rtol=1e-12, atol=1e-12, max_step=1e4, min_step=None,
                 max_steps=10_000_000, fwd=1, flip=None):
    """integrators/rk.py:2375-2549 on one trajectory; returns ((m, dim), n_acc, n_rej, status)."""
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    t_eval = np.ascontiguousarray(t_eval, dtype=np.float64)
    dim = y0.size
    lo, hi = _flip(dim, fwd, flip)
    if min_step is None:
        min_step = 10.0 * np.finfo(float).eps
    out = np.empty((t_eval.size, dim))
    na, nr = C.c_long(0), C.c_long(0)
    st = lib().hgo_dop853_dense(dim, float(mu), int(fwd), lo, hi, _p(y0), _p(t_eval), t_eval.size,
                                float(rtol), float(atol), float(max_step), float(min_step),
                                int(max_steps), _p(out), C.byref(na), C.byref(nr))
    return out, na.value, nr.value, st


def dop853_event(y0, t0, tmax, mu, ev_index, ev_offset=0.0, ev_dir=0, max_hits=1, rtol=1e-12,
                 atol=1e-12, max_step=np.inf, min_step=None, xtol=1e-12, gtol=1e-12,
                 max_steps=10_000_000, fwd=1, flip=None):
    """integrators/rk.py:2678-2803 (max_hits=1) on one trajectory."""
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    dim = y0.size
    lo, hi = _flip(dim, fwd, flip)
    if min_step is None:
        min_step = 10.0 * np.finfo(float).eps
    mh = max(int(max_hits), 1)
    hit_t = np.zeros(mh)
    hit_y = np.zeros((mh, dim))
    nh = C.c_int(0)
    t_end = C.c_double(0.0)
    y_end = np.empty(dim)
    na, nr = C.c_long(0), C.c_long(0)
    st = lib().hgo_dop853_event(dim, float(mu), int(fwd), lo, hi, _p(y0), float(t0), float(tmax),
                                float(rtol), float(atol), float(max_step), float(min_step),
                                int(max_steps), int(ev_index), float(ev_offset), int(ev_dir),
                                int(max_hits), float(xtol), float(gtol), _p(hit_t), _p(hit_y),
                                C.byref(nh), C.byref(t_end), _p(y_end), C.byref(na), C.byref(nr))
    return dict(n_hits=nh.value, hit_t=hit_t[:nh.value], hit_y=hit_y[:nh.value], t_end=t_end.value,
                y_end=y_end, n_accept=na.value, n_reject=nr.value, status=st)


def fixed_rk_event(order, y0, t_vals, mu, ev_index, ev_offset=0.0, ev_dir=0, xtol=1e-12, gtol=1e-12, fwd=1,
                   flip=None):
    """integrators/rk.py:655-718 on one trajectory: (hit, t_hit, y_hit, states)."""
    L = lib()
    if not hasattr(L, "_fre"):
        L.hgo_fixed_rk_event.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _DP, _DP, C.c_int,
                                         C.c_int, C.c_double, C.c_int, C.c_double, C.c_double, _DP, _DP, _DP]
        L.hgo_fixed_rk_event.restype = C.c_int
        L._fre = True
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    t_vals = np.ascontiguousarray(t_vals, dtype=np.float64)
    dim = y0.size
    lo, hi = _flip(dim, fwd, flip)
    states = np.full((t_vals.size, dim), np.nan)
    th = C.c_double(np.nan)
    yh = np.full(dim, np.nan)
    hit = L.hgo_fixed_rk_event(int(order), dim, float(mu), int(fwd), lo, hi, _p(y0), _p(t_vals), t_vals.size,
                               int(ev_index), float(ev_offset), int(ev_dir), float(xtol), float(gtol), _p(states),
                               C.byref(th), _p(yh))
    return hit, th.value, yh, states


def section_detect(times, states, axis, offset=0.0, direction=0, plane=(1, 4), segment_refine=50, cubic=False,
                   newton_max_iter=10, tol_on_surface=1e-6, dedup_time_tol=1e-9, dedup_point_tol=1e-6,
                   max_hits=64):
    """poincare/synodic/backend.py:458-659 on one sampled trajectory."""
    L = lib()
    if not hasattr(L, "_sec"):
        L.hgo_section_detect.argtypes = [_DP, _DP, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, _DP, _DP,
                                         _IP]
        L.hgo_section_detect.restype = C.c_int
        L._sec = True
    times = np.ascontiguousarray(times, dtype=np.float64)
    states = np.ascontiguousarray(states, dtype=np.float64)
    hit_t = np.zeros(max_hits)
    hit_y = np.zeros((max_hits, 6))
    ns = C.c_int(0)
    L.hgo_section_detect(_p(times), _p(states), len(times), int(axis), float(offset), int(direction), int(plane[0]),
                         int(plane[1]), int(segment_refine), 1 if cubic else 0, int(newton_max_iter),
                         float(tol_on_surface), float(dedup_time_tol), float(dedup_point_tol), int(max_hits),
                         _p(hit_t), _p(hit_y), C.byref(ns))
    return hit_t[:ns.value], hit_y[:ns.value]


def dop853_event_batch(y0, t0, tmax, mu, ev_index, ev_offset=0.0, ev_dir=0, max_hits=1,
                       rtol=1e-12, atol=1e-12, max_step=np.inf, min_step=None, xtol=1e-12,
                       gtol=1e-12, max_steps=10_000_000, fwd=1, flip=None, threads=None):
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    N, dim = y0.shape
    lo, hi = _flip(dim, fwd, flip)
    if min_step is None:
        min_step = 10.0 * np.finfo(float).eps
    mh = max(int(max_hits), 1)
    hit_t = np.zeros((N, mh))
    hit_y = np.zeros((N, mh, dim))
    n_hits = np.zeros(N, dtype=np.int32)
    t_end = np.zeros(N)
    y_end = np.zeros((N, dim))
    n_acc = np.zeros(N, dtype=np.int64)
    n_rej = np.zeros(N, dtype=np.int64)
    status = np.zeros(N, dtype=np.int32)
    th = threads or os.cpu_count() or 1
    lib().hgo_dop853_event_batch(dim, float(mu), int(fwd), lo, hi, N, _p(y0), float(t0), float(tmax),
                                 float(rtol), float(atol), float(max_step), float(min_step),
                                 int(max_steps), int(ev_index), float(ev_offset), int(ev_dir),
                                 int(max_hits), float(xtol), float(gtol), _p(hit_t), _p(hit_y),
                                 _p(n_hits, _IP), _p(t_end), _p(y_end), _p(n_acc, _LP),
                                 _p(n_rej, _LP), _p(status, _IP), int(th))
    return dict(hit_t=hit_t, hit_y=hit_y, n_hits=n_hits, t_end=t_end, y_end=y_end,
                n_accept=n_acc, n_reject=n_rej, status=status)
