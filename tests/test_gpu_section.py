"""GPU section detection on sampled trajectories == oracle (DEVICE mode) bit
for bit; the reference's own hits within 1e-12 (the samples are the
reference's, so only the last bit of a few squares can differ)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


@pytest.mark.parametrize("interp", ["linear", "cubic"])
@pytest.mark.parametrize("plane", ["y0dn", "xany"])
def test_gpu_section_on_dense_samples_bitexact(gpu, oracle, interp, plane):
    from hiten_gb300 import synodic
    y0 = W.section_states(257, seed=13)
    tf, m = 12.0, 600
    r = gpu.propagate_dop853(y0, 0.0, tf, MU, rtol=1e-11, atol=1e-11, n_samples=m)
    samples = r.samples
    times = np.linspace(0.0, tf, m)
    axis, off, d, pc = (("y", 0.0, -1, ("x", "vx")) if plane == "y0dn" else ("x", W.X_L1, None, ("y", "vy")))
    ht, hy, nh = synodic.detect(times, samples, section_axis=axis, section_offset=off, plane_coords=pc, direction=d,
                                interp=interp, max_hits=32)
    ht, hy, nh = ht.cpu().numpy(), hy.cpu().numpy(), nh.cpu().numpy()
    S = samples.cpu().numpy()
    oracle.set_mode(oracle.MODE_DEVICE)
    ax = synodic.AXES[axis]
    pl = (synodic.AXES[pc[0]], synodic.AXES[pc[1]])
    for i in range(len(y0)):
        rt, ry = oracle.section_detect(times, S[:, i, :], ax, off, 0 if d is None else d, pl,
                                       cubic=(interp == "cubic"), max_hits=32)
        assert nh[i] == len(rt)
        assert np.array_equal(ht[i, :nh[i]], rt) and np.array_equal(hy[i, :nh[i]], ry)
    oracle.set_mode(oracle.MODE_PYTHON)
    assert nh.sum() > 0


def test_gpu_section_vs_reference_golden(gpu):
    from hiten_gb300 import synodic
    s = np.load(os.path.join(GOLDEN, "section.npz"))
    for i in range(8):
        t, y = s[f"{i}/times"], s[f"{i}/states"]
        for kind in ("linear", "cubic"):
            ht, hy, nh = synodic.detect(t, y[:, None, :], section_axis="y", plane_coords=("x", "vx"), direction=-1,
                                        interp=kind, max_hits=32)
            rt, ry = s[f"{i}/{kind}_y0dn_t"], s[f"{i}/{kind}_y0dn_y"]
            assert int(nh[0]) == len(rt)
            assert np.max(np.abs(ht[0, :len(rt)].cpu().numpy() - rt), initial=0.0) <= 1e-12
            assert np.max(np.abs(hy[0, :len(rt)].cpu().numpy() - ry), initial=0.0) <= 1e-12
