"""Golden connection sets: the reference's own connections backend
(connections/backends.py:410-540 ``_ConnectionsBackend.run``: radius pairing,
mutual-nearest pairs, nearest neighbours on each section, segment
refinement, delta-v classification) run in pure-Python mode through
``refshim`` on seeded synthetic section point clouds.  Writes
``connections.npz``.  Run only where the reference tree is available:

    python tests/golden/make_golden_connections.py /path/to/hiten/src
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

CASES = [
    # (seed, n_u, n_s, eps, dv_tol, bal_tol, duplicates)
    (0, 300, 280, 2e-3, 0.5, 1e-2, False),
    (1, 500, 450, 5e-3, 0.2, 5e-2, False),
    (2, 200, 200, 1e-2, 1.0, 1e-1, True),    # exact duplicate points and distance ties
    (3, 1, 50, 1e-1, 1.0, 1e-1, False),      # a single unstable point (no neighbour segment)
]


def cloud(seed, n_u, n_s, dup):
    rng = np.random.default_rng(seed)
    # points along a few noisy curves on the (y, vy) section, states around them
    def curve(n, phase):
        s = rng.uniform(0, 1, n)
        y = 0.1 * np.cos(2 * np.pi * s + phase) + rng.normal(0, 2e-3, n)
        vy = 0.3 * np.sin(2 * np.pi * s + phase) + rng.normal(0, 2e-3, n)
        return np.c_[y, vy]
    pu = curve(n_u, 0.0)
    ps = curve(n_s, 0.05)
    if dup:
        pu[10] = pu[11]
        ps[5] = pu[3]
        ps[6] = pu[3]
        pu[40] = ps[40] + np.array([1e-3, 0.0])
        pu[41] = ps[40] - np.array([1e-3, 0.0])
    Xu = np.c_[np.full(n_u, 0.85), pu[:, 0], np.zeros(n_u), rng.normal(0, 0.05, n_u), pu[:, 1], rng.normal(0, 0.05, n_u)]
    Xs = np.c_[np.full(n_s, 0.85), ps[:, 0], np.zeros(n_s), rng.normal(0, 0.05, n_s), ps[:, 1], rng.normal(0, 0.05, n_s)]
    tu = rng.integers(0, 40, n_u)
    ts = rng.integers(0, 40, n_s)
    return pu, ps, Xu, Xs, tu, ts


def main(ref_src):
    sys.path.insert(0, HERE)
    import refshim
    refshim.activate(ref_src)
    from hiten.algorithms.connections.backends import _ConnectionsBackend
    from hiten.algorithms.connections.types import ConnectionsBackendRequest
    out = {}
    for c, (seed, nu, ns, eps, dvt, bt, dup) in enumerate(CASES):
        pu, ps, Xu, Xs, tu, ts = cloud(seed, nu, ns, dup)
        req = ConnectionsBackendRequest(points_u=pu, points_s=ps, states_u=Xu, states_s=Xs, traj_indices_u=tu,
                                        traj_indices_s=ts, eps=eps, dv_tol=dvt, bal_tol=bt)
        resp = _ConnectionsBackend().run(req)
        R = resp.results
        out.update({
            f"{c}/pu": pu, f"{c}/ps": ps, f"{c}/Xu": Xu, f"{c}/Xs": Xs, f"{c}/tu": tu, f"{c}/ts": ts,
            f"{c}/params": np.array([eps, dvt, bt]),
            f"{c}/kind": np.array([r.kind == "ballistic" for r in R], dtype=bool),
            f"{c}/dv": np.array([r.delta_v for r in R], dtype=float),
            f"{c}/point": np.array([r.point2d for r in R], dtype=float).reshape(-1, 2),
            f"{c}/state_u": np.array([r.state_u for r in R], dtype=float).reshape(-1, 6),
            f"{c}/state_s": np.array([r.state_s for r in R], dtype=float).reshape(-1, 6),
            f"{c}/index": np.array([[r.index_u, r.index_s, r.trajectory_index_u, r.trajectory_index_s] for r in R],
                                   dtype=np.int64).reshape(-1, 4),
            f"{c}/pairs_considered": int(resp.metadata.get("pairs_considered", 0)),
        })
        print(c, len(R), "results,", resp.metadata.get("pairs_considered"), "pairs")
    np.savez_compressed(os.path.join(HERE, "connections.npz"), n_cases=len(CASES), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path to the hiten source tree, the directory holding hiten/>")
    main(sys.argv[1])
