"""Fixed-step RK with a terminal plane event (integrators/rk.py:655-718):
GPU == oracle (DEVICE) bit for bit at 6 and 42 dimensions, and the reference's
own event times/states within 1e-12."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import stm_state
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


@pytest.mark.parametrize("order", [4, 8])
@pytest.mark.parametrize("dim", [6, 42])
def test_fixed_event_bitexact(gpu, oracle, order, dim):
    x = W.section_states(37, seed=17)
    y0 = x if dim == 6 else np.array([stm_state(v) for v in x])
    ev_index = 1 if dim == 6 else 37
    t = np.linspace(0.0, 5.0, 501)
    ev = gpu.EventSpec(index=ev_index, offset=0.0, direction=-1)
    out, ht, hy, nh = gpu.propagate_fixed_event(y0, t, MU, ev, order=order)
    ht, hy, nh = ht.cpu().numpy(), hy.cpu().numpy(), nh.cpu().numpy()
    oracle.set_mode(oracle.MODE_DEVICE)
    for i in range(len(y0)):
        hit, th, yh, _ = oracle.fixed_rk_event(order, y0[i], t, MU, ev_index, 0.0, -1)
        assert nh[i] == hit
        if hit:
            assert ht[i] == th and np.array_equal(hy[i], yh)
    oracle.set_mode(oracle.MODE_PYTHON)
    assert nh.sum() > 0


def test_fixed_event_vs_reference_golden(gpu):
    from hiten_gb300 import dynamics as D
    a = np.load(os.path.join(GOLDEN, "adaptive.npz"))
    for i in range(6):
        y0 = a[f"fixed_event/{i}/y0"]
        sol = D.propagate_dynsys(D.CR3BPSystem(MU, 6), y0, 0.0, 6.0, steps=601, method="fixed", order=8,
                                 event_fn=D.PlaneEvent(1, 0.0), event_cfg=D.EventConfig(direction=-1))
        assert abs(sol.times[-1] - a[f"fixed_event/{i}/t"][-1]) <= 1e-12
        assert np.max(np.abs(sol.states[-1] - a[f"fixed_event/{i}/states"][-1])) <= 1e-12
