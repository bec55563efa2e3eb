"""Generate the golden fixtures by running the reference itself.

The reference is pure Python + numba; numba is not installed here, so the
``refshim`` package runs the unmodified reference sources in pure-Python mode
(numba decorators become no-ops, plotting/IO modules are stubbed).  Every
fixture below is produced through the reference's own call sites:

* ``rhs.npz``       dynamics/rtbp.py:30-74 (_crtbp_accel), :167-255 (_var_equations)
* ``fixed.npz``     dynamics/base.py:346-458 (_propagate_dynsys, method='fixed'),
                    dynamics/rtbp.py:258-340 (_compute_stm, method='fixed')
* ``adaptive.npz``  _propagate_dynsys / _compute_stm with method='adaptive'
                    (DOP853 dense output), and with a terminal plane event
                    (integrators/rk.py:2678-2803)
* ``crossing.npz``  poincare/singlehit/backend.py:360 (_y_plane_crossing)
* ``halo.npz``      system/orbits/base.py:379 (orbit.correct())

Inputs come from ``hiten_gb300.workloads`` (seeded).  Run only where the
reference tree is available:

    python tests/golden/make_golden.py /path/to/hiten/src
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
REF_SRC = None


def _init(ref_src):
    sys.path.insert(0, HERE)
    import refshim
    refshim.activate(ref_src)


def _ref():
    from hiten import System
    return System.from_mu(MU)


# ----------------------------------------------------------------------------
def job_rhs(_):
    from hiten.algorithms.dynamics.rtbp import _crtbp_accel, _var_equations
    rng = np.random.default_rng(11)
    s6 = W.section_states(200, seed=3)
    s6[:, 3] = rng.uniform(-0.3, 0.3, 200)
    s6[:, 5] = rng.uniform(-0.3, 0.3, 200)
    y42 = np.zeros((200, 42))
    y42[:, :36] = rng.standard_normal((200, 36)) * 10.0 ** rng.uniform(-2, 3, (200, 36))
    y42[:, 36:] = W.section_states(200, seed=4)
    y42[:, 39] = rng.uniform(-0.3, 0.3, 200)
    d6 = np.array([_crtbp_accel(s, MU) for s in s6])
    d42 = np.array([_var_equations(0.0, y, MU) for y in y42])
    return dict(s6=s6, d6=d6, y42=y42, d42=d42)


def job_fixed(args):
    kind, i = args
    from hiten.algorithms.dynamics.base import _propagate_dynsys
    from hiten.algorithms.dynamics.rtbp import _compute_stm
    sysm = _ref()
    if kind == "rk8_42":
        y0 = W.stm_fixed_batch(1024, seed=0)[i]
        sol = _propagate_dynsys(sysm.var_dynsys, y0, 0.0, 3.0, forward=1, steps=3001, method="fixed", order=8)
        return kind, i, y0, np.asarray(sol.times), np.asarray(sol.states)[::100]
    if kind == "rk4_42":
        y0 = W.stm_fixed_batch(1024, seed=0)[100 + i]
        sol = _propagate_dynsys(sysm.var_dynsys, y0, 0.0, 1.5, forward=1, steps=601, method="fixed", order=4)
        return kind, i, y0, np.asarray(sol.times), np.asarray(sol.states)[::50]
    if kind == "rk8_42_bwd":
        x0 = W.stm_fixed_batch(1024, seed=0)[200 + i, 36:]
        x, t, phi, PHI = _compute_stm(sysm.var_dynsys, x0, 2.0, steps=401, forward=-1, method="fixed", order=8)
        return kind, i, x0, np.asarray(t), np.asarray(PHI)[::50]
    if kind in ("rk8_6", "rk6_6", "rk4_6", "rk8_6_bwd"):
        order = {"rk8_6": 8, "rk6_6": 6, "rk4_6": 4, "rk8_6_bwd": 8}[kind]
        fwd = -1 if kind.endswith("bwd") else 1
        y0 = W.section_states(64, seed=5)[i]
        sol = _propagate_dynsys(sysm.dynsys, y0, 0.0, 2.0, forward=fwd, steps=801, method="fixed", order=order)
        return kind, i, y0, np.asarray(sol.times), np.asarray(sol.states)[::20]
    raise ValueError(kind)


def job_adaptive(args):
    kind, i = args
    from hiten.algorithms.dynamics.base import _propagate_dynsys
    from hiten.algorithms.dynamics.rtbp import _compute_stm
    from hiten.algorithms.types.configs import EventConfig
    sysm = _ref()
    if kind == "stm_halo":
        fwd = 1 if i == 0 else -1
        x, t, phi, PHI = _compute_stm(sysm.var_dynsys, W.HALO_L1_AZ02_X0, W.HALO_L1_AZ02_T, steps=40,
                                      forward=fwd, method="adaptive", order=8)
        return kind, i, W.HALO_L1_AZ02_X0.copy(), np.asarray(t), np.asarray(PHI)
    if kind == "dense6":
        y0 = W.section_states(64, seed=6)[i]
        sol = _propagate_dynsys(sysm.dynsys, y0, 0.0, 4.0, forward=1, steps=101, method="adaptive", order=8,
                                rtol=1e-11, atol=1e-11)
        return kind, i, y0, np.asarray(sol.times), np.asarray(sol.states)
    if kind in ("manifold_fwd", "manifold_bwd"):
        # halo-state perturbations propagated to the x = 1 - mu plane
        rng = np.random.default_rng(100 + i)
        y0 = W.HALO_L1_AZ02_X0 + rng.uniform(-1e-5, 1e-5, 6)
        fwd = 1 if kind == "manifold_fwd" else -1
        off = float(1 - MU)

        def g(t, y):
            return float(y[0] - off)

        sol = _propagate_dynsys(sysm.dynsys, y0, 0.0, 8.0, forward=fwd, steps=2, method="adaptive", order=8,
                                flip_indices=slice(0, 6), rtol=1e-12, atol=1e-12, event_fn=g,
                                event_cfg=EventConfig(direction=0, terminal=True))
        return kind, i, y0, np.asarray(sol.times), np.asarray(sol.states)
    if kind == "fixed_event":
        y0 = W.section_states(64, seed=9)[i]

        def g(t, y):
            return float(y[1])

        sol = _propagate_dynsys(sysm.dynsys, y0, 0.0, 6.0, forward=1, steps=601, method="fixed", order=8,
                                event_fn=g, event_cfg=EventConfig(direction=-1, terminal=True))
        return kind, i, y0, np.asarray(sol.times), np.asarray(sol.states)
    if kind == "section":
        y0 = W.section_states(64, seed=7)[i]

        def g(t, y):
            return float(y[1])

        sol = _propagate_dynsys(sysm.dynsys, y0, 0.0, 20.0, forward=1, steps=2, method="adaptive", order=8,
                                rtol=1e-11, atol=1e-11, event_fn=g,
                                event_cfg=EventConfig(direction=-1, terminal=True))
        return kind, i, y0, np.asarray(sol.times), np.asarray(sol.states)
    raise ValueError(kind)


def job_section(i):
    """Sampled DOP853 trajectory + the synodic detection backend (linear and cubic)."""
    from hiten.algorithms.dynamics.base import _propagate_dynsys
    from hiten.algorithms.poincare.synodic.backend import _SynodicDetectionBackend
    sysm = _ref()
    y0 = W.section_states(64, seed=8)[i]
    sol = _propagate_dynsys(sysm.dynsys, y0, 0.0, 12.0, forward=1, steps=600, method="adaptive", order=8,
                            rtol=1e-11, atol=1e-11)
    times, states = np.asarray(sol.times), np.asarray(sol.states)
    out = {"times": times, "states": states}
    be = _SynodicDetectionBackend()
    for kind in ("linear", "cubic"):
        for name, normal, off, direction, plane in (("y0dn", [0, 1, 0, 0, 0, 0], 0.0, -1, ("x", "vx")),
                                                     ("xany", [1, 0, 0, 0, 0, 0], float(W.X_L1 if y0[0] < 1 else
                                                                                        W.X_L2), None, ("y", "vy"))):
            hits = be.detect_on_trajectory(times, states, normal=np.array(normal, float), offset=off,
                                           plane_coords=plane, interp_kind=kind, segment_refine=50,
                                           tol_on_surface=1e-6, dedup_time_tol=1e-9, dedup_point_tol=1e-6,
                                           max_hits_per_traj=None, newton_max_iter=10, direction=direction)
            out[f"{kind}_{name}_t"] = np.array([h.time for h in hits], dtype=float)
            out[f"{kind}_{name}_y"] = np.array([h.state for h in hits], dtype=float).reshape(-1, 6)
            out[f"{kind}_{name}_off"] = off
    return i, out


def job_crossing(i):
    from hiten.algorithms.poincare.singlehit.backend import _y_plane_crossing
    sysm = _ref()
    rng = np.random.default_rng(200 + i)
    y0 = W.HALO_L1_AZ02_X0 + np.array([rng.uniform(-1e-3, 1e-3), 0, rng.uniform(-1e-3, 1e-3), 0,
                                        rng.uniform(-1e-3, 1e-3), 0])
    t, s = _y_plane_crossing(dynsys=sysm.dynsys, x0=y0)
    return i, y0, t, np.asarray(s)


def job_halo(args):
    point, az, zen = args
    sysm = _ref()
    L = sysm.get_libration_point(point)
    orb = L.create_orbit("halo", amplitude_z=az, zenith=zen)
    guess = np.asarray(orb.initial_state, dtype=float).copy()
    res = orb.correct()
    iters = getattr(res, "iterations", -1)
    return point, az, zen, guess, np.asarray(orb.initial_state, dtype=float), float(orb.period), int(iters if iters is not None else -1)


def main(ref_src):
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(8, os.cpu_count() or 1), initializer=_init, initargs=(ref_src,)) as pool:
        r_rhs = pool.apply_async(job_rhs, (0,))
        fixed_jobs = ([("rk8_42", i) for i in range(6)] + [("rk4_42", i) for i in range(2)]
                      + [("rk8_42_bwd", i) for i in range(2)]
                      + [(k, i) for k in ("rk8_6", "rk6_6", "rk4_6", "rk8_6_bwd") for i in range(3)])
        r_fixed = pool.map_async(job_fixed, fixed_jobs)
        ad_jobs = ([("stm_halo", 0), ("stm_halo", 1)] + [("dense6", i) for i in range(4)]
                   + [(k, i) for k in ("manifold_fwd", "manifold_bwd") for i in range(4)]
                   + [("section", i) for i in range(12)] + [("fixed_event", i) for i in range(6)])
        r_ad = pool.map_async(job_adaptive, ad_jobs)
        r_cross = pool.map_async(job_crossing, range(6))
        r_sec = pool.map_async(job_section, range(8))
        halo_jobs = [(p, az, z) for p in (1, 2) for az in (0.05, 0.2) for z in ("southern", "northern")]
        r_halo = pool.map_async(job_halo, halo_jobs)

        np.savez_compressed(os.path.join(HERE, "rhs.npz"), mu=MU, **r_rhs.get())
        out = {}
        for kind, i, y0, t, s in r_fixed.get():
            out[f"{kind}/{i}/y0"] = y0
            out[f"{kind}/{i}/t"] = t
            out[f"{kind}/{i}/states"] = s
        np.savez_compressed(os.path.join(HERE, "fixed.npz"), mu=MU, **out)
        out = {}
        for kind, i, y0, t, s in r_ad.get():
            out[f"{kind}/{i}/y0"] = y0
            out[f"{kind}/{i}/t"] = t
            out[f"{kind}/{i}/states"] = s
        np.savez_compressed(os.path.join(HERE, "adaptive.npz"), mu=MU, **out)
        cr = r_cross.get()
        np.savez_compressed(os.path.join(HERE, "crossing.npz"), mu=MU,
                            y0=np.array([c[1] for c in cr]), t=np.array([c[2] for c in cr]),
                            state=np.array([c[3] for c in cr]))
        sec = {}
        for i, d in r_sec.get():
            for k, v in d.items():
                sec[f"{i}/{k}"] = v
        np.savez_compressed(os.path.join(HERE, "section.npz"), mu=MU, **sec)
        hr = r_halo.get()
        np.savez_compressed(os.path.join(HERE, "halo.npz"), mu=MU,
                            point=np.array([h[0] for h in hr]), az=np.array([h[1] for h in hr]),
                            zenith=np.array([h[2] for h in hr]), guess=np.array([h[3] for h in hr]),
                            x0=np.array([h[4] for h in hr]), period=np.array([h[5] for h in hr]),
                            iterations=np.array([h[6] for h in hr]))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path to the hiten source tree, the directory holding hiten/>")
    main(sys.argv[1])
