"""Golden halo families: the reference's own orbit continuation
(system/orbits/base.py:410 ``orbit.generate()`` ->
continuation/backends/pc.py:42-166 with the secant or natural-parameter
stepper, continuation/stepping/) run in pure-Python mode through
``refshim``, from seed orbits corrected by the reference.  Writes
``family.npz``.  Run only where the reference tree is available:

    python tests/golden/make_golden_family.py /path/to/hiten/src
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from hiten_gb300 import workloads as W  # noqa: E402

MU = W.MU_EM

# (libration point, Az of the seed, zenith, stepper, step in z, max members)
FAMILIES = [
    (1, 0.2, "southern", "secant", 0.004, 4),
    (2, 0.1, "northern", "natural", -0.006, 4),
    (1, 0.05, "southern", "secant", 0.25, 3),   # a step too long: rejections and halving
]


def _init(ref_src):
    sys.path.insert(0, HERE)
    import refshim
    refshim.activate(ref_src)


def job_family(i):
    from hiten import System
    from hiten.algorithms.continuation.config import OrbitContinuationConfig
    from hiten.algorithms.continuation.options import OrbitContinuationOptions
    from hiten.algorithms.types.states import SynodicState
    point, az, zen, stepper, step, members = FAMILIES[i]
    L = System.from_mu(MU).get_libration_point(point)
    orb = L.create_orbit("halo", amplitude_z=az, zenith=zen)
    orb.correct()
    seed = np.asarray(orb.initial_state, dtype=float).copy()
    seed_period = float(orb.period)
    orb.continuation_config = OrbitContinuationConfig(state=(SynodicState.Z,), stepper=stepper)
    z0 = seed[2]
    opts = OrbitContinuationOptions(target=([z0 - 1.0], [z0 + 1.0]), step=(step,), max_members=members,
                                    max_retries_per_step=50)
    res = orb.generate(options=opts)
    fam = np.array([np.asarray(m.initial_state, dtype=float) for m in res.family])
    periods = np.array([np.nan if m.period is None else float(m.period) for m in res.family])
    params = np.array([np.asarray(p, dtype=float) for p in res.parameter_values])
    return (i, seed, seed_period, fam, periods, params, int(res.accepted_count), int(res.rejected_count),
            int(res.iterations))


def main(ref_src):
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(FAMILIES), initializer=_init, initargs=(ref_src,)) as pool:
        rows = pool.map(job_family, range(len(FAMILIES)))
    out = {"mu": MU}
    for i, seed, seed_period, fam, periods, params, acc, rej, it in rows:
        point, az, zen, stepper, step, members = FAMILIES[i]
        out.update({f"{i}/seed": seed, f"{i}/seed_period": seed_period, f"{i}/family": fam,
                    f"{i}/periods": periods, f"{i}/params": params, f"{i}/accepted": acc, f"{i}/rejected": rej,
                    f"{i}/iterations": it, f"{i}/stepper": stepper, f"{i}/step": step, f"{i}/members": members,
                    f"{i}/point": point})
    np.savez_compressed(os.path.join(HERE, "family.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path to the hiten source tree, the directory holding hiten/>")
    main(sys.argv[1])
