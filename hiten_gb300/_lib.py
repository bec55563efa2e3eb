"""ctypes binding of ``libhitengpu.so`` (C ABI declared in include/hitengpu.h).

There is no CPU fallback: importing the binding on a machine without the
library or without a CUDA device raises, and every non-zero call status is
turned into an exception.
"""
import ctypes as C
import os
import threading

from . import build as _build

HG_OK = 0
HG_MAX_STEPS = 1
HG_STEP_UNDERFLOW = 2
HG_NONFINITE = 3
HG_NEWTON_DIVERGED = 4
HG_EVENT_NOT_FOUND = 5
HG_LINE_SEARCH_FAILED = 6
HG_SYNC_TIMEOUT = 7
HG_ERR_ARGS = 10
HG_ERR_CUDA = 11
HG_ERR_NO_DEVICE = 12
HG_ERR_TIMEOUT = 13

STATUS_NAMES = {0: "OK", 1: "MAX_STEPS", 2: "STEP_UNDERFLOW", 3: "NONFINITE", 4: "NEWTON_DIVERGED",
                5: "EVENT_NOT_FOUND", 6: "LINE_SEARCH_FAILED", 7: "SYNC_TIMEOUT", 10: "ERR_ARGS", 11: "ERR_CUDA", 12: "ERR_NO_DEVICE", 13: "ERR_TIMEOUT"}

EXPORTED = ("hg_create", "hg_destroy", "hg_last_error_string", "hg_version", "hg_propagate_fixed",
            "hg_propagate_dop853", "hg_probe_fp64_peak", "hg_propagate_dop853_noalloc", "hg_set_tuning",
            "hg_get_tuning", "hg_section_detect", "hg_trajectory_filters", "hg_propagate_fixed_event",
            "hg_dop853_segmented_workspace_bytes", "hg_propagate_dop853_segmented",
            "hg_propagate_dop853_scheduled", "hg_get_counter", "hg_radius_best", "hg_nearest_neighbor", "hg_connection_refine",
            "hg_newton_opts_default", "hg_correct_halo", "hg_serve_config_default", "hg_serve_create",
            "hg_serve_destroy", "hg_serve_submit", "hg_serve_poll", "hg_serve_wait", "hg_serve_fetch",
            "hg_serve_cancel", "hg_serve_stats", "hg_selftest_bounded_wait", "hg_host_pow", "hg_reserve",
            "hg_reserve_correct", "hg_points_workspace_bytes", "hg_correct_halo_graph_workspace_bytes",
            "hg_correct_halo_graph")
HG_COUNTER_KERNEL_LAUNCHES = 1
HG_COUNTER_ALLOCATIONS = 2
HG_RUNNING = -1
HG_TUNE_BLOCK_THREADS = 1
HG_TUNE_DOP853_LANES_D6 = 2
HG_TUNE_SEG_STEPS = 3
HG_TUNE_SPREAD = 4
HG_TUNE_LANES_D42 = 5
HG_TUNE_SM_CAPACITY = 6
HG_TUNE_REFINE_POOL_MB = 7


class HitenGpuError(RuntimeError):
    """A hitengpu call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"hitengpu error {code} ({STATUS_NAMES.get(code, '?')}): {msg}")
        self.code = code


class hg_event(C.Structure):
    _fields_ = [("index", C.c_int), ("offset", C.c_double), ("direction", C.c_int), ("max_hits", C.c_int),
                ("xtol", C.c_double), ("gtol", C.c_double)]


class hg_dop853_opts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("max_step", C.c_double), ("min_step", C.c_double),
                ("max_steps", C.c_longlong), ("fwd", C.c_int), ("flip_lo", C.c_int), ("flip_hi", C.c_int)]


class hg_newton_opts(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_attempts", C.c_int), ("max_delta", C.c_double),
                ("alpha_reduction", C.c_double), ("min_alpha", C.c_double), ("armijo_c", C.c_double),
                ("cond_threshold", C.c_double), ("event_rtol", C.c_double), ("event_atol", C.c_double),
                ("stm_rtol", C.c_double), ("stm_atol", C.c_double), ("steps", C.c_int)]


class hg_serve_config(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget_bytes", C.c_longlong), ("max_concurrent", C.c_int),
                ("staging_bytes", C.c_longlong), ("pool_slots", C.c_int), ("seg_steps", C.c_int)]


class hg_config(C.Structure):
    _fields_ = [("device", C.c_int)]


_P = C.c_void_p
_lib = None
_lock = threading.Lock()


def load(build_if_missing=True):
    """Load (building first if needed) the shared library; no fallback."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing and _build.stale():
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"hitengpu library missing at {path}; run hiten_gb300.build.build()")
        L = C.CDLL(path)
        L.hg_create.argtypes = [C.POINTER(hg_config), C.POINTER(_P)]
        L.hg_create.restype = C.c_int
        L.hg_destroy.argtypes = [_P]
        L.hg_destroy.restype = C.c_int
        L.hg_last_error_string.argtypes = [_P]
        L.hg_last_error_string.restype = C.c_char_p
        L.hg_version.restype = C.c_char_p
        L.hg_propagate_fixed.argtypes = [_P, C.c_double, C.c_int, C.c_int, C.c_int, _P, C.c_longlong, _P, C.c_int,
                                         C.c_int, _P, C.c_longlong, C.c_int, C.c_int, C.c_int, _P, _P]
        L.hg_propagate_fixed.restype = C.c_int
        L.hg_propagate_dop853.argtypes = [_P, C.c_double, C.c_int, C.c_int, _P, C.c_longlong, _P, _P, C.c_double,
                                          C.c_double, C.POINTER(hg_dop853_opts), C.POINTER(hg_event), C.c_int,
                                          C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]
        L.hg_propagate_dop853.restype = C.c_int
        L.hg_propagate_dop853_noalloc.argtypes = [C.c_double, C.c_int, C.c_int, _P, C.c_longlong, _P, _P,
                                                  C.c_double, C.c_double, C.POINTER(hg_dop853_opts),
                                                  C.POINTER(hg_event), C.c_int, C.c_int, _P, _P, _P, _P, _P, _P,
                                                  _P, _P, _P, _P]
        L.hg_propagate_dop853_noalloc.restype = C.c_int
        L.hg_section_detect.argtypes = [C.c_int, C.c_int, _P, C.c_longlong, _P, C.c_longlong, C.c_int, C.c_double,
                                        C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                        C.c_double, C.c_double, C.c_int, _P, _P, _P, _P, _P]
        L.hg_section_detect.restype = C.c_int
        L.hg_trajectory_filters.argtypes = [C.c_int, C.c_int, _P, C.c_longlong, C.c_double, _P, _P, _P, _P]
        L.hg_trajectory_filters.restype = C.c_int
        L.hg_propagate_fixed_event.argtypes = [_P, C.c_double, C.c_int, C.c_int, C.c_int, _P, C.c_longlong, _P,
                                               C.c_int, C.c_int, _P, C.c_longlong, C.c_int, C.c_int, C.c_int,
                                               C.POINTER(hg_event), _P, _P, _P, _P, _P]
        L.hg_propagate_fixed_event.restype = C.c_int
        L.hg_dop853_segmented_workspace_bytes.argtypes = [C.c_int, C.c_int, C.c_int]
        L.hg_dop853_segmented_workspace_bytes.restype = C.c_longlong
        L.hg_propagate_dop853_segmented.argtypes = (L.hg_propagate_dop853.argtypes[:-1]
                                                    + [C.c_int, C.c_int, C.c_int, _P, C.c_longlong, _P])
        L.hg_propagate_dop853_segmented.restype = C.c_int
        L.hg_propagate_dop853_scheduled.argtypes = L.hg_propagate_dop853.argtypes[:-1] + [_P, C.c_longlong, _P]
        L.hg_propagate_dop853_scheduled.restype = C.c_int
        L.hg_set_tuning.argtypes = [_P, C.c_int, C.c_int]
        L.hg_set_tuning.restype = C.c_int
        L.hg_get_tuning.argtypes = [_P, C.c_int, C.POINTER(C.c_int)]
        L.hg_get_tuning.restype = C.c_int
        L.hg_points_workspace_bytes.argtypes = [C.c_int]
        L.hg_points_workspace_bytes.restype = C.c_longlong
        L.hg_radius_best.argtypes = [C.c_int, _P, _P, C.c_int, _P, _P, C.c_double, C.c_double, _P, _P, _P, _P,
                                     C.c_longlong, _P]
        L.hg_radius_best.restype = C.c_int
        L.hg_nearest_neighbor.argtypes = [C.c_int, _P, _P, C.c_double, _P, _P, C.c_longlong, _P]
        L.hg_nearest_neighbor.restype = C.c_int
        L.hg_connection_refine.argtypes = [C.c_int, _P, _P, _P, _P, _P, C.c_int, _P, _P, C.c_int, _P, _P, _P, _P, _P,
                                           _P]
        L.hg_connection_refine.restype = C.c_int
        L.hg_newton_opts_default.argtypes = [C.POINTER(hg_newton_opts)]
        L.hg_newton_opts_default.restype = None
        L.hg_correct_halo.argtypes = [_P, C.c_double, C.c_int, _P, C.c_longlong, _P, _P, _P, _P,
                                      C.POINTER(hg_newton_opts), _P]
        L.hg_correct_halo.restype = C.c_int
        L.hg_serve_config_default.argtypes = [C.POINTER(hg_serve_config)]
        L.hg_serve_config_default.restype = None
        L.hg_serve_create.argtypes = [C.POINTER(hg_serve_config), C.POINTER(_P)]
        L.hg_serve_destroy.argtypes = [_P]
        L.hg_serve_submit.argtypes = [_P, C.c_double, C.c_int, C.c_int, _P, C.c_double, C.c_double,
                                      C.POINTER(hg_dop853_opts), C.POINTER(hg_event), C.POINTER(C.c_longlong)]
        L.hg_serve_poll.argtypes = [_P, C.c_longlong, C.POINTER(C.c_int)]
        L.hg_serve_wait.argtypes = [_P, C.c_longlong, C.c_double]
        L.hg_serve_fetch.argtypes = [_P, C.c_longlong, _P, _P, _P, _P, _P, _P, _P, _P]
        L.hg_serve_cancel.argtypes = [_P, C.c_longlong]
        L.hg_serve_stats.argtypes = [_P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                     C.POINTER(C.c_longlong)]
        for f in ("hg_serve_create", "hg_serve_destroy", "hg_serve_submit", "hg_serve_poll", "hg_serve_wait",
                  "hg_serve_fetch", "hg_serve_cancel", "hg_serve_stats"):
            getattr(L, f).restype = C.c_int
        L.hg_get_counter.argtypes = [_P, C.c_int, C.POINTER(C.c_longlong)]
        L.hg_reserve.argtypes = [_P, C.c_int, C.c_int, C.c_int]
        L.hg_reserve.restype = C.c_int
        L.hg_reserve_correct.argtypes = [_P, C.c_int]
        L.hg_reserve_correct.restype = C.c_int
        L.hg_correct_halo_graph_workspace_bytes.argtypes = [C.c_int]
        L.hg_correct_halo_graph_workspace_bytes.restype = C.c_longlong
        L.hg_correct_halo_graph.argtypes = [_P, C.c_double, C.c_int, _P, C.c_longlong, _P, _P, _P, _P,
                                            C.POINTER(hg_newton_opts), _P, C.c_longlong, _P]
        L.hg_correct_halo_graph.restype = C.c_int
        L.hg_selftest_bounded_wait.argtypes = [_P, C.c_int, _P, _P]
        L.hg_selftest_bounded_wait.restype = C.c_int
        L.hg_host_pow.argtypes = [C.c_longlong, _P, C.c_double, _P]
        L.hg_host_pow.restype = None
        L.hg_get_counter.restype = C.c_int
        L.hg_probe_fp64_peak.argtypes = [_P, C.POINTER(C.c_double)]
        L.hg_probe_fp64_peak.restype = C.c_int
        _lib = L
        return L


class Handle:
    """Owns one ``hg_handle`` (per device)."""

    def __init__(self, device=0):
        self.lib = load()
        h = _P()
        cfg = hg_config(int(device))
        rc = self.lib.hg_create(C.byref(cfg), C.byref(h))
        if rc != HG_OK:
            raise HitenGpuError(rc, "hg_create failed (no CUDA device?)")
        self.ptr = h
        self.device = int(device)

    def check(self, rc):
        if rc != HG_OK:
            msg = self.lib.hg_last_error_string(self.ptr)
            raise HitenGpuError(rc, msg.decode() if msg else "")

    def set_tuning(self, key, value):
        self.check(self.lib.hg_set_tuning(self.ptr, int(key), int(value)))

    def get_tuning(self, key):
        v = C.c_int(0)
        self.check(self.lib.hg_get_tuning(self.ptr, int(key), C.byref(v)))
        return v.value

    def kernel_launches(self):
        """Kernels launched through this handle so far."""
        v = C.c_longlong(0)
        self.check(self.lib.hg_get_counter(self.ptr, HG_COUNTER_KERNEL_LAUNCHES, C.byref(v)))
        return v.value

    def allocations(self):
        """Device and pinned-host allocations made for this handle so far."""
        v = C.c_longlong(0)
        self.check(self.lib.hg_get_counter(self.ptr, HG_COUNTER_ALLOCATIONS, C.byref(v)))
        return v.value

    def reserve(self, max_n, dim, max_hits):
        """Size the event-refinement pool for calls up to these sizes (hg_reserve)."""
        self.check(self.lib.hg_reserve(self.ptr, int(max_n), int(dim), int(max_hits)))

    def reserve_correct(self, max_orbits):
        """Size the corrector's buffers for up to max_orbits orbits (hg_reserve_correct)."""
        self.check(self.lib.hg_reserve_correct(self.ptr, int(max_orbits)))

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.hg_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def handle(device=0):
    """This thread's handle for a device (created on first use).  A handle
    owns the lane-refill scratch of the calls made through it, so each host
    thread gets its own: calls from different threads on different streams
    never share scratch."""
    hs = getattr(_tls, "handles", None)
    if hs is None:
        hs = _tls.handles = {}
    h = hs.get(device)
    if h is None:
        h = Handle(device)
        hs[device] = h
    return h
