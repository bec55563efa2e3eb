"""Golden manifold seeding, acceptance filters and orbit stability, produced
by running the reference itself (pure-Python mode through ``refshim``).
Writes ``manifold.npz``:

* the L1 southern halo with Az = 0.2 corrected by ``orbit.correct()``; for its
  stable and unstable manifolds (direction 'positive'):
  - ``_ManifoldDynamicsService.compute_stm(steps=2000)``
    (types/services/manifold.py:215-245): xx, tt, PHI;
  - the eigen-decomposition of the monodromy and the real eigenvector the
    service follows (NN = 1, :347-367; algorithms/linalg/backend.py:196-260);
  - ``_compute_manifold_section`` (:470-537) for a seeded sample of
    (fraction, displacement) pairs;
* for four of the stable seeds, the trajectory ``compute_manifold`` propagates
  (``_propagate_dynsys``, DOP853 backward, dense samples, :377-396), its
  minimum distances to both primaries (:398-402) and
  ``_max_rel_energy_error`` (common/energy.py:27-74);
* ``orbit.compute_stability()`` (types/services/orbits.py:664-687) of eight
  corrected halo orbits (L1/L2, Az 0.05/0.2, both zeniths): indices,
  eigenvalues, eigenvectors, and the monodromy matrix it decomposed.

Run only where the reference tree is available:

    python tests/golden/make_golden_manifold.py /path/to/hiten/src
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
N_SEEDS = 24
N_TRAJ = 4
TRAJ_FRACTION = 0.25   # integration_fraction of the sampled trajectories (tf = pi / 2)
TRAJ_DT = 2e-3


def _init(ref_src):
    sys.path.insert(0, HERE)
    import refshim
    refshim.activate(ref_src)


def _sample():
    rng = np.random.default_rng(31)
    fr = rng.uniform(0.0, 1.0, N_SEEDS)
    disp = np.exp(rng.uniform(np.log(1e-7), np.log(1e-5), N_SEEDS))
    return fr, disp


def job_manifold(stable):
    from hiten import System
    from hiten.algorithms.common.energy import _max_rel_energy_error
    from hiten.algorithms.dynamics.base import _propagate_dynsys
    sysm = System.from_mu(MU)
    orb = sysm.get_libration_point(1).create_orbit("halo", amplitude_z=0.2, zenith="southern")
    orb.correct()
    man = orb.manifold(stable=stable, direction="positive")
    svc = man.dynamics
    xx, tt, phi_T, PHI = svc.compute_stm(steps=2000)
    sn, un, _ = svc.eigenvalues
    Ws, Wu, _ = svc.eigenvectors
    _, s_real = svc.stability.get_real_eigenvectors(Ws, sn)
    _, u_real = svc.stability.get_real_eigenvectors(Wu, un)
    eigvec = (s_real if stable else u_real)[:, 0]
    fr, disp = _sample()
    seeds = np.array([svc._compute_manifold_section(period=orb.period, fraction=f, displacement=d, xx=xx, tt=tt,
                                                    PHI=PHI, eigvec=eigvec).astype(np.float64)
                      for f, d in zip(fr, disp)])
    out = {"x0": np.asarray(orb.initial_state, dtype=float), "period": float(orb.period), "xx": xx, "tt": tt,
           "PHI": PHI, "phi_T": phi_T, "sn": sn, "un": un, "Ws": Ws, "Wu": Wu, "eigvec": eigvec,
           "fractions": fr, "displacements": disp, "seeds": seeds, "direction": int(svc.direction),
           "forward": int(svc.forward)}
    if stable:
        mu = MU
        tf = TRAJ_FRACTION * 2 * np.pi
        steps = max(int(abs(tf) / TRAJ_DT) + 1, 100)
        states, r1m, r2m, de = [], [], [], []
        for x0W in seeds[:N_TRAJ]:
            sol = _propagate_dynsys(dynsys=svc.dynsys, state0=x0W, t0=0.0, tf=tf, forward=svc.forward, steps=steps,
                                    method="adaptive", order=8, flip_indices=slice(0, 6))
            st = sol.states
            x, y, z = st[:, 0], st[:, 1], st[:, 2]
            r1 = np.sqrt((x + mu) ** 2 + y ** 2 + z ** 2)
            r2 = np.sqrt((x - 1 + mu) ** 2 + y ** 2 + z ** 2)
            states.append(st)
            r1m.append(r1.min())
            r2m.append(r2.min())
            de.append(_max_rel_energy_error(st, mu))
        dist_m = sysm.distance * 1e3
        out.update(traj_states=np.array(states), traj_min_r1=np.array(r1m), traj_min_r2=np.array(r2m),
                   traj_max_rel_energy=np.array(de), traj_tf=tf, traj_steps=steps,
                   primary_radius_nd=sysm.primary.radius / dist_m, secondary_radius_nd=sysm.secondary.radius / dist_m)
    return stable, out


def job_stability(args):
    from hiten import System
    point, az, zen = args
    orb = System.from_mu(MU).get_libration_point(point).create_orbit("halo", amplitude_z=az, zenith=zen)
    orb.correct()
    nu, w, V = orb.dynamics.compute_stability()
    from hiten.algorithms.dynamics.rtbp import _compute_stm
    _, _, Phi, _ = _compute_stm(orb.dynamics.var_dynsys, orb.initial_state, orb.period)
    return (point, az, zen, np.asarray(orb.initial_state, dtype=float), float(orb.period), np.asarray(nu),
            np.asarray(w), np.asarray(V), np.asarray(Phi))


def main(ref_src):
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(8, os.cpu_count() or 1), initializer=_init, initargs=(ref_src,)) as pool:
        r_man = pool.map_async(job_manifold, (True, False))
        st_jobs = [(p, az, z) for p in (1, 2) for az in (0.05, 0.2) for z in ("southern", "northern")]
        r_st = pool.map_async(job_stability, st_jobs)
        out = {"mu": MU}
        for stable, d in r_man.get():
            tag = "stable" if stable else "unstable"
            out.update({f"{tag}/{k}": v for k, v in d.items()})
        rows = r_st.get()
        out.update(stab_point=np.array([r[0] for r in rows]), stab_az=np.array([r[1] for r in rows]),
                   stab_zenith=np.array([r[2] for r in rows]), stab_x0=np.array([r[3] for r in rows]),
                   stab_period=np.array([r[4] for r in rows]), stab_nu=np.array([r[5] for r in rows]),
                   stab_eigvals=np.array([r[6] for r in rows]), stab_eigvecs=np.array([r[7] for r in rows]),
                   stab_monodromy=np.array([r[8] for r in rows]))
    np.savez_compressed(os.path.join(HERE, "manifold.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path to the hiten source tree, the directory holding hiten/>")
    main(sys.argv[1])
