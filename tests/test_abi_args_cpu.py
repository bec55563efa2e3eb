"""Argument checks of the handle-free C-ABI entry points, on the host: bad
sizes and missing buffers give HG_ERR_ARGS and empty batches HG_OK before any
device work, so these calls need no GPU.  Every call here is invalid or empty:
the buffers are host memory and must never reach a kernel."""
import ctypes as C

import pytest

from hiten_gb300 import _lib


@pytest.fixture(scope="module")
def L():
    return _lib.load()


def _buf(n=8, t=C.c_double):
    return (t * n)()


def test_connection_search_args(L):
    x, i = _buf(), _buf(t=C.c_int)
    ok, bad = _lib.HG_OK, _lib.HG_ERR_ARGS
    # negative sizes, NaN or negative eps / coord_max
    assert L.hg_radius_best(-1, x, x, 1, x, x, 0.1, 1.0, i, i, x, None, 0, None) == bad
    assert L.hg_radius_best(1, x, x, -1, x, x, 0.1, 1.0, i, i, x, None, 0, None) == bad
    assert L.hg_radius_best(1, x, x, 1, x, x, -0.1, 1.0, i, i, x, None, 0, None) == bad
    assert L.hg_radius_best(1, x, x, 1, x, x, float("nan"), 1.0, i, i, x, None, 0, None) == bad
    assert L.hg_radius_best(1, x, x, 1, x, x, 0.1, -1.0, i, i, x, None, 0, None) == bad
    # missing query or output buffers; reference buffers only when nr > 0
    assert L.hg_radius_best(1, None, x, 1, x, x, 0.1, 1.0, i, i, x, None, 0, None) == bad
    assert L.hg_radius_best(1, x, x, 1, x, x, 0.1, 1.0, None, i, x, None, 0, None) == bad
    assert L.hg_radius_best(1, x, x, 1, None, x, 0.1, 1.0, i, i, x, None, 0, None) == bad
    # an empty query set is done before anything touches the device
    assert L.hg_radius_best(0, None, None, 5, None, None, 0.1, 1.0, None, None, None, None, 0, None) == ok
    assert L.hg_nearest_neighbor(-1, x, x, 1.0, i, None, 0, None) == bad
    assert L.hg_nearest_neighbor(3, x, x, -1.0, i, None, 0, None) == bad
    assert L.hg_nearest_neighbor(3, None, x, 1.0, i, None, 0, None) == bad
    assert L.hg_nearest_neighbor(3, x, x, 1.0, None, None, 0, None) == bad
    assert L.hg_nearest_neighbor(0, None, None, 1.0, None, None, 0, None) == ok
    # a caller workspace smaller than hg_points_workspace_bytes(n) is refused up front
    w = _buf(64, C.c_double)
    assert L.hg_points_workspace_bytes(3) == 256 and L.hg_points_workspace_bytes(-1) == -1
    assert L.hg_nearest_neighbor(3, x, x, 1.0, i, w, 255, None) == bad
    assert L.hg_radius_best(1, x, x, 40, x, x, 0.1, 1.0, i, i, x, w, 256, None) == bad
    b = _buf(t=C.c_ubyte)
    assert L.hg_connection_refine(-1, i, i, i, i, b, 1, x, x, 1, x, x, x, x, x, None) == bad
    assert L.hg_connection_refine(1, i, i, i, i, b, -1, x, x, 1, x, x, x, x, x, None) == bad
    assert L.hg_connection_refine(1, None, i, i, i, b, 1, x, x, 1, x, x, x, x, x, None) == bad
    assert L.hg_connection_refine(1, i, i, i, i, None, 1, x, x, 1, x, x, x, x, x, None) == bad
    assert L.hg_connection_refine(1, i, i, i, i, b, 1, x, x, 1, x, x, x, x, None, None) == bad
    assert L.hg_connection_refine(0, None, None, None, None, None, 0, None, None, 0, None, None, None, None, None,
                                  None) == ok


def test_section_and_filter_args(L):
    x, i = _buf(64), _buf(t=C.c_int)
    ok, bad = _lib.HG_OK, _lib.HG_ERR_ARGS

    def det(N=1, m=2, ld=1, tld=0, axis=1, pu=0, pv=3, direction=0, refine=5, max_hits=2, newton=3, samples=x):
        return L.hg_section_detect(N, m, samples, ld, x, tld, axis, 0.0, direction, pu, pv, refine, 1, newton, 1e-9,
                                   1e-9, 1e-9, max_hits, x, x, i, None, None)

    assert det(N=-1) == bad
    assert det(ld=0) == bad  # ld < N
    assert det(N=2, ld=2, tld=1) == bad  # per-trajectory times need tld >= N
    assert det(axis=6) == bad and det(pu=-1) == bad and det(pv=6) == bad
    assert det(direction=2) == bad and det(refine=0) == bad and det(max_hits=0) == bad and det(newton=-1) == bad
    assert det(samples=None) == bad
    assert det(N=0, ld=0, samples=None) == ok
    assert L.hg_trajectory_filters(-1, 2, x, 1, 0.01, x, x, x, None) == bad
    assert L.hg_trajectory_filters(1, 0, x, 1, 0.01, x, x, x, None) == bad
    assert L.hg_trajectory_filters(2, 2, x, 1, 0.01, x, x, x, None) == bad  # ld < N
    assert L.hg_trajectory_filters(1, 2, None, 1, 0.01, x, x, x, None) == bad
    assert L.hg_trajectory_filters(0, 2, None, 0, 0.01, None, None, None, None) == ok


def test_noalloc_propagation_args(L):
    x, i = _buf(64), _buf(t=C.c_int)
    bad = _lib.HG_ERR_ARGS
    o = _lib.hg_dop853_opts()
    o.rtol = o.atol = 1e-12
    o.max_step, o.min_step, o.max_steps = 1e4, 1e-15, 1000
    o.fwd, o.flip_lo, o.flip_hi = 1, 0, 0

    def run(dim=6, N=1, ld=1, opts=o, y0=x, n_samples=0, ys=None):
        return L.hg_propagate_dop853_noalloc(0.01, dim, N, y0, ld, None, None, 0.0, 1.0, C.byref(opts) if opts else None,
                                             None, n_samples, 0, ys, x, x, x, x, i, i, i, i, None)

    assert run(dim=7) == bad
    assert run(N=-1) == bad and run(N=2, ld=1) == bad
    assert run(opts=None) == bad and run(y0=None) == bad
    assert run(n_samples=1) == bad and run(n_samples=4, ys=None) == bad
    o.flip_lo, o.flip_hi = 3, 2
    assert run() == bad
    o.flip_lo, o.flip_hi, o.rtol = 0, 0, -1.0
    assert run() == bad
    o.rtol, o.max_steps = 1e-12, 0
    assert run() == bad


def test_native_server_host_checks(L):
    """The request server's defaults and argument checks; on a machine
    without a device its creation fails with HG_ERR_NO_DEVICE (no worker)."""
    import torch
    c = _lib.hg_serve_config()
    L.hg_serve_config_default(C.byref(c))
    assert (c.device, c.hbm_budget_bytes, c.max_concurrent, c.staging_bytes, c.pool_slots, c.seg_steps) == \
        (0, 8 << 30, 4, 1 << 30, 32768, 16)
    out = C.c_void_p(123)
    assert L.hg_serve_create(C.byref(c), None) == _lib.HG_ERR_ARGS
    for field, bad in (("max_concurrent", 0), ("max_concurrent", 65), ("hbm_budget_bytes", 0), ("staging_bytes", 0),
                       ("pool_slots", 31), ("seg_steps", 0)):
        d = _lib.hg_serve_config()
        L.hg_serve_config_default(C.byref(d))
        setattr(d, field, bad)
        assert L.hg_serve_create(C.byref(d), C.byref(out)) == _lib.HG_ERR_ARGS
        assert out.value is None  # cleared on every failure
        out = C.c_void_p(123)
    assert L.hg_serve_destroy(None) == _lib.HG_OK
    y, i = _buf(6), C.c_longlong(0)
    o = _lib.hg_dop853_opts()
    assert L.hg_serve_submit(None, 0.01, 6, 1, y, 0.0, 1.0, C.byref(o), None, C.byref(i)) == _lib.HG_ERR_ARGS
    if not torch.cuda.is_available():
        assert L.hg_serve_create(C.byref(c), C.byref(out)) == _lib.HG_ERR_NO_DEVICE
        assert out.value is None
