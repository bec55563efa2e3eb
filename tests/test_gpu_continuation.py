"""Halo-family continuation on the GPU against the reference's own families
(tests/golden/family.npz): same accepted / rejected counts and iterations,
members and periods within the corrected-orbit tolerance (1e-10)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_gpu_families_match_reference(gpu):
    from hiten_gb300 import continuation as Cn
    fam = np.load(os.path.join(GOLDEN, "family.npz"))
    mu = float(fam["mu"])
    seeds = np.array([fam[f"{i}/seed"] for i in range(3)])
    periods = np.array([float(fam[f"{i}/seed_period"]) for i in range(3)])
    opts = []
    for i in range(3):
        z0 = seeds[i, 2]
        opts.append(Cn.ContinuationOptions(step=(float(fam[f"{i}/step"]),), target=([z0 - 1.0], [z0 + 1.0]),
                                           max_members=int(fam[f"{i}/members"]), stepper=str(fam[f"{i}/stepper"])))
    res = Cn.continue_halo_families(seeds, periods, mu, options=opts)
    for i, r in enumerate(res):
        assert r.accepted_count == int(fam[f"{i}/accepted"])
        assert r.rejected_count == int(fam[f"{i}/rejected"])
        assert r.iterations == int(fam[f"{i}/iterations"])
        assert np.max(np.abs(np.array(r.family) - fam[f"{i}/family"])) <= 1e-10
        assert np.max(np.abs(np.array(r.periods) - fam[f"{i}/periods"])) <= 1e-10
