"""Generate the golden trajectories in tests/golden/ from the CPU FP64 oracle.

The Julia reference cannot run on this machine, so the fixtures come from the
oracle (oracle/kb_oracle.cpp), whose sunset is pinned against numpy's
rfftn/irfftn and whose three engines agree with each other; see
tests/test_oracle.py. Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ENGINE_FULL, ENGINE_OCTANT, Oracle  # noqa: E402

# config 1 of the benchmark list: Ns=16, O(4), lambda=1, m=1, dt=0.1, 200 steps,
# full memory window (NstepsinMemory = Nsteps + 2 = 202), thermal T=2, RNone
C1 = dict(name="c1_ns16_m202", Ns=16, M=202, N=4, lam=1.0, dt=0.1, T=2.0, steps=200, engine=ENGINE_OCTANT)
# small full-lattice (CPUfull) case with a wrapping ring
SMALL = dict(name="small_ns8_m10", Ns=8, M=10, N=4, lam=2.0, dt=0.1, T=2.0, steps=40, engine=ENGINE_FULL)


def generate(cfg):
    o = Oracle(cfg["Ns"], 3, M=cfg["M"], N=cfg["N"], dt=cfg["dt"], lam=cfg["lam"], mass2=1.0, mass=1.0,
               engine=cfg["engine"], nthreads=4)
    rep, k2, deg = o.orbits()
    n0 = 1.0 / (np.exp(np.sqrt(k2 + 1.0) / cfg["T"]) - 1.0)
    o.init_occupation(n0, 1.0)
    ts, scal, nsnap, tsnap = [], [], [], []
    m = o.measure(2)
    ts.append(2)
    scal.append([m[k] for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")])
    for t in range(3, 3 + cfg["steps"]):
        o.step(t)
        m = o.measure(t)
        ts.append(t)
        scal.append([m[k] for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")])
        if (t - 2) % 20 == 0 or t == 2 + cfg["steps"]:
            nsnap.append(m["n"])
            tsnap.append(t)
    t = 2 + cfg["steps"]
    tmin, tmax = o.window()
    tps = np.arange(tmin, t + 1, max(1, (t - tmin) // 40))
    Frow = np.array([o.F(t, tp) for tp in tps])
    rrow = np.array([o.rho(t, tp) for tp in tps])
    out = os.path.join(HERE, cfg["name"] + ".npz")
    np.savez_compressed(out, t=np.array(ts), scalars=np.array(scal), n_t=np.array(tsnap), n=np.array(nsnap),
                        F_last_row=Frow, rho_last_row=rrow, tps=tps, tmin=tmin, k2=k2, deg=deg, n0=n0,
                        cfg=np.array([cfg["Ns"], cfg["M"], cfg["N"], cfg["lam"], cfg["dt"], cfg["T"], cfg["steps"]]))
    print("wrote", out)


if __name__ == "__main__":
    for c in (SMALL, C1):
        generate(c)
