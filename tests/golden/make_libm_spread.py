"""How much the reference's own results depend on the C library's pow.

The reference (numba, fastmath off) computes its fractional powers -- the
DOP853 step controller's err**(-1/9), err_prev**(0.4/9), err**(-1/8)
(integrators/utils.py:242,247,280) and the Jacobian's r2**1.5, r2**2.5
(dynamics/rtbp.py:119-122,230-231) -- with the platform's libm pow, which is
not correctly rounded.  On x86-64, glibc picks its pow at load time: an FMA
build on CPUs with FMA and AVX2, a non-FMA build otherwise; the two differ in
about 0.07 % of calls for these exponents.  This script runs the CPU oracle
in the reference's arithmetic (numba lowering of integer powers, libm pow)
once under each glibc variant (GLIBC_TUNABLES masks FMA/AVX2 for the second)
on seeded samples of the synodic-section workload (65536-state set, DOP853
1e-11, t = 20, up to 8 decreasing y = 0 crossings) and of the stable-manifold
workload (t = -8, terminal x = 1 - mu), and writes ``libm_spread.npz``:
the crossings and end states of each run.

Run on an x86-64 host with glibc >= 2.28 and an FMA-capable CPU:

    python tests/golden/make_libm_spread.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
N_SECTION = 512
N_MANIFOLD = 512


def child(out_path):
    sys.path.insert(0, REPO)
    from hiten_gb300 import manifold as M
    from hiten_gb300 import workloads as W
    from oracle import hgo
    mu = W.MU_EM
    hgo.set_mode(hgo.MODE_NUMBA)
    y0 = W.section_states(65536, seed=0)
    idx = np.sort(np.random.default_rng(11).choice(len(y0), N_SECTION, replace=False))
    sec = hgo.dop853_event_batch(y0[idx], 0.0, 20.0, mu, 1, 0.0, -1, 8, rtol=1e-11, atol=1e-11, max_step=1e4)
    # manifold seeds from the orbit's STM grid in the reference's arithmetic
    T = W.HALO_L1_AZ02_T
    PHI, _, _, _ = hgo.dop853_dense(W.identity_stm_state(W.HALO_L1_AZ02_X0)[0], np.linspace(0.0, T, 2000), mu,
                                    fwd=-1, flip=(36, 42))
    v = M.stable_eigvec(PHI[-1, :36].reshape(6, 6), stable=True)
    phases, disp = W.manifold_grid(512, 32, seed=0)
    seeds = M.seeds(-np.linspace(0.0, T, 2000), PHI, T, phases, disp, v, direction=1)
    midx = np.sort(np.random.default_rng(12).choice(len(seeds), N_MANIFOLD, replace=False))
    man = hgo.dop853_event_batch(seeds[midx], 0.0, 8.0, mu, 0, 1 - mu, 0, 1, max_step=1e4, fwd=-1, flip=(0, 6))
    out = {"section_idx": idx, "section_y0": y0[idx], "manifold_idx": midx, "manifold_y0": seeds[midx]}
    for tag, r in (("section", sec), ("manifold", man)):
        for k in ("hit_t", "hit_y", "n_hits", "y_end", "t_end", "n_accept", "n_reject"):
            out[f"{tag}_{k}"] = r[k]
    np.savez(out_path, **out)


def main():
    runs = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, env_extra in (("fma", {}), ("nofma", {"GLIBC_TUNABLES": "glibc.cpu.hwcaps=-AVX2,-FMA"})):
            path = os.path.join(tmp, f"{name}.npz")
            env = dict(os.environ, **env_extra)
            subprocess.check_call([sys.executable, os.path.abspath(__file__), "--child", path], env=env)
            runs[name] = dict(np.load(path))
    out = {}
    for name, d in runs.items():
        for k, v in d.items():
            if k.endswith("_idx") or k.endswith("_y0"):
                out[k] = v
            else:
                out[f"{name}/{k}"] = v
    out["note"] = json.dumps({"host": os.uname().machine, "glibc": os.confstr("CS_GNU_LIBC_VERSION")})
    np.savez_compressed(os.path.join(HERE, "libm_spread.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) == 3 and sys.argv[1] == "--child":
        child(sys.argv[2])
    else:
        main()
