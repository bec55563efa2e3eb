"""hg_propagate_dop853_noalloc -- the DOP853 entry point for callers that
cannot allocate device memory (no handle; its lane-refill counter lives in a
static device array) -- must give the same results as hg_propagate_dop853,
bit for bit, on consecutive calls that reuse that static scratch.

The batch is larger than the resident lanes, so finished lanes claim new
trajectories through the static counter; a stale counter from the previous
call would skip or repeat trajectories and show up as a mismatch.  This file
sorts last so that a run stopping at the first failure has run everything
else already; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


def _noalloc_call(lib, y0_soa, N, tmax, ev, outs, stream):
    import torch
    from hiten_gb300 import _lib
    opts = _lib.hg_dop853_opts(1e-11, 1e-11, 1e4, 10 * np.finfo(float).eps, 100000, 1, 0, 6)
    evs = _lib.hg_event(ev.index, ev.offset, ev.direction, ev.max_hits, ev.xtol, ev.gtol)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    rc = lib.hg_propagate_dop853_noalloc(MU, 6, N, p(y0_soa), N, None, None, 0.0, float(tmax), C.byref(opts),
                                         C.byref(evs), 0, 0, None, p(outs["y_end"]), p(outs["t_end"]),
                                         p(outs["hit_t"]), p(outs["hit_y"]), p(outs["n_hits"]),
                                         p(outs["n_acc"]), p(outs["n_rej"]), p(outs["status"]), stream)
    torch.cuda.synchronize()
    return rc


def test_noalloc_matches_handle_entry_point_twice(gpu):
    import torch
    from hiten_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    N = 60000  # more trajectories than resident lanes: the refill counter is used
    y0 = W.section_states(N, seed=21)
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=3)
    ref = gpu.propagate_dop853(y0, 0.0, 0.7, MU, rtol=1e-11, atol=1e-11, event=ev, device=dev)
    torch.cuda.synchronize()
    y0_soa = torch.as_tensor(y0, device=dev).t().contiguous()
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for call in range(2):
        outs = {"y_end": torch.full((6, N), np.nan, dtype=torch.float64, device=dev),
                "t_end": torch.full((N,), np.nan, dtype=torch.float64, device=dev),
                "hit_t": torch.full((3, N), np.nan, dtype=torch.float64, device=dev),
                "hit_y": torch.full((3, 6, N), np.nan, dtype=torch.float64, device=dev),
                "n_hits": torch.full((N,), -1, dtype=torch.int32, device=dev),
                "n_acc": torch.full((N,), -1, dtype=torch.int32, device=dev),
                "n_rej": torch.full((N,), -1, dtype=torch.int32, device=dev),
                "status": torch.full((N,), -1, dtype=torch.int32, device=dev)}
        assert _noalloc_call(lib, y0_soa, N, 0.7, ev, outs, stream) == _lib.HG_OK, f"call {call}"
        assert torch.equal(outs["y_end"].t(), ref.y_end), f"call {call}: end states differ"
        assert torch.equal(outs["t_end"], ref.t_end)
        assert torch.equal(outs["n_acc"], ref.n_accept) and torch.equal(outs["n_rej"], ref.n_reject)
        assert torch.equal(outs["n_hits"], ref.n_hits) and torch.equal(outs["status"], ref.status)
        k = ref.n_hits.cpu().numpy()
        ht, hy = outs["hit_t"].t().cpu().numpy(), outs["hit_y"].permute(2, 0, 1).cpu().numpy()
        rt, ry = ref.hit_t.cpu().numpy(), ref.hit_y.cpu().numpy()
        for i in np.nonzero(k)[0][:2000]:
            assert np.array_equal(ht[i, :k[i]], rt[i, :k[i]]) and np.array_equal(hy[i, :k[i]], ry[i, :k[i]])


def _noalloc_generic(lib, dim, y0_soa, N, tmax, ev, outs, stream, hit_t=True):
    import torch
    from hiten_gb300 import _lib
    opts = _lib.hg_dop853_opts(1e-11, 1e-11, 1e4, 10 * np.finfo(float).eps, 100000, 1, 0, 6)
    evs = _lib.hg_event(ev.index, ev.offset, ev.direction, ev.max_hits, ev.xtol, ev.gtol)
    p = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    rc = lib.hg_propagate_dop853_noalloc(MU, dim, N, p(y0_soa), N, None, None, 0.0, float(tmax), C.byref(opts),
                                         C.byref(evs), 0, 0, None, p(outs["y_end"]), p(outs["t_end"]),
                                         p(outs["hit_t"]) if hit_t else None, p(outs["hit_y"]),
                                         p(outs["n_hits"]), p(outs["n_acc"]), p(outs["n_rej"]),
                                         p(outs["status"]), stream)
    torch.cuda.synchronize()
    return rc


def _outs(dim, N, max_hits, dev):
    import torch
    return {"y_end": torch.full((dim, N), np.nan, dtype=torch.float64, device=dev),
            "t_end": torch.full((N,), np.nan, dtype=torch.float64, device=dev),
            "hit_t": torch.full((max_hits, N), np.nan, dtype=torch.float64, device=dev),
            "hit_y": torch.full((max_hits, dim, N), np.nan, dtype=torch.float64, device=dev),
            "n_hits": torch.full((N,), -1, dtype=torch.int32, device=dev),
            "n_acc": torch.full((N,), -1, dtype=torch.int32, device=dev),
            "n_rej": torch.full((N,), -1, dtype=torch.int32, device=dev),
            "status": torch.full((N,), -1, dtype=torch.int32, device=dev)}


def test_noalloc_stm_matches_handle_entry_point_twice(gpu):
    """The 42-dim (state + STM) kernel through the entry point, with an
    x = 0.84 event: more trajectories than its resident lanes, so the static refill
    counter is used; two calls in a row equal the handle entry point."""
    import torch
    from hiten_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    N = 6000
    y0 = W.stm_fixed_batch(N, seed=22)
    ev = gpu.EventSpec(index=36, offset=0.84, direction=0, max_hits=2)
    ref = gpu.propagate_dop853(y0, 0.0, 0.6, MU, rtol=1e-11, atol=1e-11, event=ev, device=dev)
    torch.cuda.synchronize()
    y0_soa = torch.as_tensor(y0, device=dev).t().contiguous()
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    assert int(ref.n_hits.sum()) > 0
    for call in range(2):
        outs = _outs(42, N, 2, dev)
        assert _noalloc_generic(lib, 42, y0_soa, N, 0.6, ev, outs, stream) == _lib.HG_OK, f"call {call}"
        assert torch.equal(outs["y_end"].t(), ref.y_end), f"call {call}: end states differ"
        assert torch.equal(outs["t_end"], ref.t_end)
        assert torch.equal(outs["n_acc"], ref.n_accept) and torch.equal(outs["n_rej"], ref.n_reject)
        assert torch.equal(outs["n_hits"], ref.n_hits) and torch.equal(outs["status"], ref.status)
        k = ref.n_hits.cpu().numpy()
        ht, hy = outs["hit_t"].t().cpu().numpy(), outs["hit_y"].permute(2, 0, 1).cpu().numpy()
        rt, ry = ref.hit_t.cpu().numpy(), ref.hit_y.cpu().numpy()
        for i in np.nonzero(k)[0]:
            assert np.array_equal(ht[i, :k[i]], rt[i, :k[i]]) and np.array_equal(hy[i, :k[i]], ry[i, :k[i]])


def test_noalloc_argument_rules_match_handle_entry_point(gpu):
    """Both entry points accept and reject the same arguments: null optional
    outputs are accepted, an event without hit buffers and a bad sample count
    are rejected."""
    import torch
    from hiten_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    N = 64
    y0 = torch.as_tensor(W.section_states(N, seed=3), device=dev).t().contiguous()
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    hh = C.c_void_p()
    assert lib.hg_create(C.byref(_lib.hg_config(0)), C.byref(hh)) == _lib.HG_OK
    opts = _lib.hg_dop853_opts(1e-11, 1e-11, 1e4, 1e-15, 100000, 1, 0, 6)
    evs = _lib.hg_event(1, 0.0, -1, 2, 1e-12, 1e-12)
    o = _outs(6, N, 2, dev)
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    cases = {
        "no outputs, no event": dict(ev=None, m=0, ys=None, ye=None, ht=None, hy=None, nh=None),
        "end states only": dict(ev=None, m=0, ys=None, ye=P(o["y_end"]), ht=None, hy=None, nh=None),
        "event without hit_t": dict(ev=C.byref(evs), m=0, ys=None, ye=P(o["y_end"]), ht=None, hy=P(o["hit_y"]),
                                    nh=P(o["n_hits"])),
        "one sample": dict(ev=None, m=1, ys=P(o["y_end"]), ye=None, ht=None, hy=None, nh=None),
        "samples without buffer": dict(ev=None, m=3, ys=None, ye=None, ht=None, hy=None, nh=None),
    }
    try:
        for name, c in cases.items():
            args = (MU, 6, N, P(y0), N, None, None, 0.0, 0.3, C.byref(opts), c["ev"], c["m"], 0, c["ys"], c["ye"],
                    None, c["ht"], c["hy"], c["nh"], None, None, None, stream)
            rc_n = lib.hg_propagate_dop853_noalloc(*args)
            rc_h = lib.hg_propagate_dop853(hh, *args)
            torch.cuda.synchronize()
            assert rc_n == rc_h, f"{name}: no-alloc {rc_n}, handle {rc_h}"
    finally:
        lib.hg_destroy(hh)


def test_noalloc_rejects_oversized_batch(gpu):
    from hiten_gb300 import _lib
    lib = _lib.load()
    opts = _lib.hg_dop853_opts(1e-11, 1e-11, 1e4, 1e-15, 10, 1, 0, 6)
    too_many = (1 << 30) + 1
    rc = lib.hg_propagate_dop853_noalloc(MU, 6, too_many, C.c_void_p(16), too_many, None, None, 0.0, 1.0,
                                         C.byref(opts), None, 0, 0, None, None, None, None, None, None, None,
                                         None, None, None)
    assert rc == _lib.HG_ERR_ARGS
