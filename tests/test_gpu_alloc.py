"""The allocation contract of the C ABI: once a handle has been reserved for
the sizes a caller uses (hg_reserve, hg_reserve_correct), repeated
propagation, event-refinement, correction and scheduled calls allocate no
device or pinned memory (HG_COUNTER_ALLOCATIONS stays where it was), and the
connection searches allocate nothing when given a workspace.  Without a
reservation a larger call grows the handle's buffer once, and calls of that
size after it allocate nothing."""
import numpy as np
import pytest

from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


def _guesses(n):
    from hiten_gb300 import halo
    pt, az, zen = W.halo_guess_params(n, seed=3)
    return np.concatenate([halo.third_order_guess(MU, 1, az[pt == 1], zen[pt == 1]),
                           halo.third_order_guess(MU, 2, az[pt == 2], zen[pt == 2])])


def test_reserved_handle_allocates_nothing(gpu):
    import torch
    from hiten_gb300 import _lib, corrector
    H = _lib.handle(0)
    H.reserve(4096, 42, 8)
    H.reserve_correct(64)
    a0 = H.allocations()
    sec = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
    y6 = W.section_states(4096, seed=7)
    y42 = W.stm_fixed_batch(512, seed=1)
    g = _guesses(64)
    for _ in range(3):
        gpu.propagate_dop853(y6, 0.0, 2.0, MU, rtol=1e-11, atol=1e-11, event=sec, scheduled=False)
        gpu.propagate_dop853(y6, 0.0, 2.0, MU, rtol=1e-11, atol=1e-11, event=sec, scheduled=True)
        gpu.propagate_dop853(y42, 0.0, 0.4, MU, event=gpu.EventSpec(index=36, offset=0.84, max_hits=2),
                             scheduled=False)
        gpu.propagate_dop853(y42, 0.0, 0.4, MU, n_samples=5)
        gpu.propagate_fixed(y42, np.linspace(0.0, 0.2, 21), MU, order=8, out_every=10)
        res = corrector.correct_halo_native(g, MU)
        assert (res.status == 0).sum() >= 60
        torch.cuda.synchronize()
        assert H.allocations() == a0


def test_unreserved_refinement_pool_grows_once(gpu):
    """A fresh handle: the first event call larger than its pool grows the
    pool once; the same call again allocates nothing."""
    import ctypes as C

    import torch
    from hiten_gb300 import _lib
    H = _lib.Handle(0)
    try:
        a0 = H.allocations()
        assert a0 == 2  # hg_create: refill counters and the pinned live-count word
        dev = torch.device("cuda", 0)
        N = 2000
        y0 = torch.as_tensor(W.section_states(N, seed=9), device=dev).t().contiguous()
        outs = [torch.empty((6, N), dtype=torch.float64, device=dev), torch.empty(N, dtype=torch.float64, device=dev),
                torch.empty((4, N), dtype=torch.float64, device=dev), torch.empty((4, 6, N), dtype=torch.float64,
                                                                               device=dev)]
        ints = [torch.empty(N, dtype=torch.int32, device=dev) for _ in range(4)]
        opts = _lib.hg_dop853_opts(1e-11, 1e-11, 1e4, 1e-15, 100000, 1, 0, 6)
        ev = _lib.hg_event(1, 0.0, -1, 4, 1e-12, 1e-12)
        p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        st = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        counts = []
        for _ in range(3):
            H.check(H.lib.hg_propagate_dop853(H.ptr, MU, 6, N, p(y0), N, None, None, 0.0, 1.5, C.byref(opts),
                                              C.byref(ev), 0, 0, None, *(p(t) for t in outs),
                                              *(p(t) for t in ints), st))
            torch.cuda.synchronize()
            counts.append(H.allocations())
        assert counts == [a0 + 1, a0 + 1, a0 + 1]
    finally:
        H.close()


def test_connection_searches_with_workspace_allocate_nothing(gpu):
    """The searches with a caller workspace give the same results as without
    one (where they allocate their FP32 copy per call)."""
    import ctypes as C

    import torch
    from hiten_gb300 import _lib
    L = _lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(4)
    n = 5000
    pts = torch.as_tensor(rng.uniform(-1, 1, (2, n)), device=dev)
    q = torch.as_tensor(rng.uniform(-1, 1, (2, 3000)), device=dev)
    ws = torch.empty(L.hg_points_workspace_bytes(n), dtype=torch.uint8, device=dev)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    st = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    res = []
    for w, wb in ((None, 0), (p(ws), ws.numel())):
        cnt = torch.empty(3000, dtype=torch.int32, device=dev)
        bi = torch.empty(3000, dtype=torch.int32, device=dev)
        bd = torch.empty(3000, dtype=torch.float64, device=dev)
        nn = torch.empty(n, dtype=torch.int32, device=dev)
        assert L.hg_radius_best(3000, p(q[0]), p(q[1]), n, p(pts[0]), p(pts[1]), 0.02, 1.0, p(cnt), p(bi), p(bd),
                                w, wb, st) == _lib.HG_OK
        assert L.hg_nearest_neighbor(n, p(pts[0]), p(pts[1]), 1.0, p(nn), w, wb, st) == _lib.HG_OK
        torch.cuda.synchronize()
        res.append((cnt.cpu(), bi.cpu(), bd.cpu(), nn.cpu()))
    for a, b in zip(*res):
        assert torch.equal(a, b)
