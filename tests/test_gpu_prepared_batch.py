"""The prepared DOP853 batch (propagate.Dop853Batch) gives the bits of
propagate_dop853 with the same arguments, run after run on new states (the
hit arrays reset to NaN each run), scheduled and single-pass."""
import numpy as np
import pytest
import torch

from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


@pytest.mark.parametrize("scheduled", [True, False])
def test_prepared_batch_equals_propagate(gpu, scheduled):
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=4)
    b = gpu.Dop853Batch(3000, 6, 0.0, 6.0, MU, rtol=1e-11, atol=1e-11, event=ev, scheduled=scheduled)
    for seed in (1, 2):
        y = torch.as_tensor(W.section_states(3000, seed=seed), device="cuda")
        got = b.run(y)
        ref = gpu.propagate_dop853(y, 0.0, 6.0, MU, rtol=1e-11, atol=1e-11, event=ev, scheduled=scheduled)
        for f in ("y_end", "t_end", "n_accept", "n_reject", "status", "n_hits"):
            assert torch.equal(getattr(got, f), getattr(ref, f)), (seed, f)
        for f in ("hit_t", "hit_y"):
            assert np.array_equal(getattr(got, f).cpu().numpy(), getattr(ref, f).cpu().numpy(), equal_nan=True), f


def test_prepared_batch_checks_the_shape(gpu):
    b = gpu.Dop853Batch(10, 6, 0.0, 1.0, MU)
    with pytest.raises(ValueError):
        b.run(np.zeros((11, 6)))


def test_prepared_batch_from_pinned_host_states(gpu):
    """Host input (pinned): the same bits as the device-resident input."""
    ev = gpu.EventSpec(index=0, offset=1.0 - MU, direction=0, max_hits=1)
    b = gpu.Dop853Batch(500, 6, 0.0, 3.0, MU, fwd=-1, flip=(0, 6), event=ev)
    y = W.section_states(500, seed=4)
    dev = b.run(torch.as_tensor(y, device="cuda"))
    d = {f: getattr(dev, f).clone() for f in ("y_end", "t_end", "n_accept", "n_hits")}
    host = b.run(torch.as_tensor(y).pin_memory())
    for f, v in d.items():
        assert torch.equal(getattr(host, f), v), f


def test_prepared_batch_to_host_reads_every_output(gpu):
    """to_host() reads the whole output arena back in one copy: every field
    on the host equals the device result's, run after run."""
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=3)
    b = gpu.Dop853Batch(700, 6, 0.0, 4.0, MU, rtol=1e-11, atol=1e-11, event=ev)
    for seed in (5, 6):
        r = b.run(torch.as_tensor(W.section_states(700, seed=seed)).pin_memory())
        h = b.to_host()
        for f in ("y_end", "t_end", "n_accept", "n_reject", "status", "n_hits", "hit_t", "hit_y"):
            dv, hv = getattr(r, f), getattr(h, f)
            assert hv.device.type == "cpu" and hv.shape == dv.shape, (seed, f)
            assert np.array_equal(hv.numpy(), dv.cpu().numpy(), equal_nan=True), (seed, f)
