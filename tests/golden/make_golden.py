"""Generate the golden trajectories in tests/golden/ from the CPU FP64 oracle.

The Julia reference cannot run on this machine, so the fixtures come from the
oracle (oracle/kb_oracle.cpp), whose sunset is pinned against numpy's
rfftn/irfftn and whose three engines agree with each other; see
tests/test_oracle.py. Run from the repository root:

    python tests/golden/make_golden.py                 # every fixture
    python tests/golden/make_golden.py c2 c3_ns48      # a selection

Fixtures at the stated sizes of the benchmark configurations:
  c1_ns16_m202  config 1: Ns=16, lambda=1, dt=0.1, 200 steps, full window, thermal T=2
  c2_ns32_m400  config 2: Ns=32, lambda=4, dt=0.05, M=400, 1000 steps, tsunami state
                initialised with the gap mass (TwoPIScalar_Initialization.jl:309-314)
  c3_ns48_m442, c3_ns24_m164
                config 3: the first Ns=48 and the first Ns=24 run of the 64-run batch
                drawn with seed 12345 (the benchmark's draw), 500 steps each, so the
                window wraps
  c5_ns64_m128  the headline lattice of config 5 (Ns=64, lambda=2, dt=0.05, tsunami state with
                the gap mass) on a 128-step window, 200 steps (the window wraps)
  c4_adjoint_ns24_m300
                config 4: loss = 8 radial-shell means of n(p, 302) + E(302) at Ns=24,
                M=300, 300 steps; forward-mode dual-number derivatives along lambda,
                m^2 and one initial-occupation direction (orc_dual_loss)
Trajectory fixtures store every step's scalars (time, E, E_pot, E_kin, E_mem, M2),
n per orbit every 50 steps (20 for short runs) and sampled F, rho rows at the last
time.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ENGINE_FULL, ENGINE_OCTANT, Oracle  # noqa: E402
from oracle.pyoracle import dual_loss  # noqa: E402

NTHREADS = int(os.environ.get("KB_GOLDEN_THREADS", str(os.cpu_count() or 4)))


def c3_draw(seed=12345, nruns=64):
    """The 64-run batch of config 3: Ns from {16,24,32,48}, lambda U[0.5,8], T U[0.5,3],
    M U{100..500}, in the order of the benchmark's draw."""
    rng = np.random.default_rng(seed)
    runs = []
    for _ in range(nruns):
        runs.append(dict(Ns=int(rng.choice([16, 24, 32, 48])), lam=float(rng.uniform(0.5, 8.0)),
                         T=float(rng.uniform(0.5, 3.0)), M=int(rng.integers(100, 501))))
    return runs


def _c3(index):
    r = c3_draw()[index]
    return dict(name=f"c3_ns{r['Ns']}_m{r['M']}", Ns=r["Ns"], M=r["M"], N=4, lam=r["lam"], dt=0.05, T=r["T"],
                steps=500, engine=ENGINE_OCTANT, init="thermal", every=50, batch_index=index)


# config 1 of the benchmark list: Ns=16, O(4), lambda=1, m=1, dt=0.1, 200 steps,
# full memory window (NstepsinMemory = Nsteps + 2 = 202), thermal T=2, RNone
C1 = dict(name="c1_ns16_m202", Ns=16, M=202, N=4, lam=1.0, dt=0.1, T=2.0, steps=200, engine=ENGINE_OCTANT,
          init="thermal", every=20)
# small full-lattice (CPUfull) case with a wrapping ring
SMALL = dict(name="small_ns8_m10", Ns=8, M=10, N=4, lam=2.0, dt=0.1, T=2.0, steps=40, engine=ENGINE_FULL,
             init="thermal", every=20)
C2 = dict(name="c2_ns32_m400", Ns=32, M=400, N=4, lam=4.0, dt=0.05, T=0.0, steps=1000, engine=ENGINE_OCTANT,
          init="tsunami", every=50)
C3A = _c3(10)   # Ns=48, M=442
C3B = _c3(7)    # Ns=24, M=164
# the headline lattice (Ns=64, lambda=2, tsunami with the gap mass) on a 128-step window
# that wraps: the full M=1000 history (52 GB FP64) is beyond a fixture run
C5S = dict(name="c5_ns64_m128", Ns=64, M=128, N=4, lam=2.0, dt=0.05, T=0.0, steps=200, engine=ENGINE_OCTANT,
           init="tsunami", every=50, rows=10)
C4 = dict(name="c4_adjoint_ns24_m300", Ns=24, M=300, N=4, lam=2.0, dt=0.05, mass2=1.0, t_final=302, nbumps=8,
          seed=12345)


def occupation(cfg, k2):
    if cfg["init"] == "thermal":
        return 1.0 / (np.exp(np.sqrt(k2 + 1.0) / cfg["T"]) - 1.0)
    return 5.0 * np.exp(-((np.sqrt(k2) - 1.0) ** 2) / (2 * 0.2 ** 2))


def generate(cfg):
    t_start = time.time()
    o = Oracle(cfg["Ns"], 3, M=cfg["M"], N=cfg["N"], dt=cfg["dt"], lam=cfg["lam"], mass2=1.0, mass=1.0,
               engine=cfg["engine"], nthreads=NTHREADS)
    rep, k2, deg = o.orbits()
    n0 = occupation(cfg, k2)
    # tsunami: initialize! takes the gap mass (Initialization.jl:309-314); otherwise disc.Mass
    init_mass = o.gap_mass(n0, 0.5) if cfg["init"] == "tsunami" else 1.0
    o.init_occupation(n0, init_mass)
    ts, scal, nsnap, tsnap = [], [], [], []
    m = o.measure(2)
    ts.append(2)
    scal.append([m[k] for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")])
    for t in range(3, 3 + cfg["steps"]):
        o.step(t)
        m = o.measure(t)
        ts.append(t)
        scal.append([m[k] for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")])
        if (t - 2) % cfg["every"] == 0 or t == 2 + cfg["steps"]:
            nsnap.append(m["n"])
            tsnap.append(t)
    t = 2 + cfg["steps"]
    tmin, tmax = o.window()
    tps = np.arange(tmin, t + 1, max(1, (t - tmin) // cfg.get("rows", 40)))
    if tps[-1] != t:
        tps = np.append(tps, t)
    Frow = np.array([o.F(t, tp) for tp in tps])
    rrow = np.array([o.rho(t, tp) for tp in tps])
    o.close()
    out = os.path.join(HERE, cfg["name"] + ".npz")
    np.savez_compressed(out, t=np.array(ts), scalars=np.array(scal), n_t=np.array(tsnap), n=np.array(nsnap),
                        F_last_row=Frow, rho_last_row=rrow, tps=tps, tmin=tmin, k2=k2, deg=deg, n0=n0,
                        init_mass=init_mass, batch_index=cfg.get("batch_index", -1),
                        cfg=np.array([cfg["Ns"], cfg["M"], cfg["N"], cfg["lam"], cfg["dt"], cfg["T"], cfg["steps"]]))
    print(f"wrote {out} ({time.time() - t_start:.0f} s, {NTHREADS} threads)", flush=True)


def generate_adjoint(cfg):
    """Config 4 loss and its exact derivatives along lambda, m^2 and one occupation
    direction, from the dual-number restatement of the oracle (single thread)."""
    t_start = time.time()
    o = Oracle(cfg["Ns"], 3, M=cfg["M"], N=cfg["N"], dt=cfg["dt"], lam=cfg["lam"], mass2=cfg["mass2"])
    _, k2, deg = o.orbits()
    o.close()
    p = np.sqrt(k2)
    nb = cfg["nbumps"]
    # bump basis and shell weights of the adjoint workload (kb2pi.adjoint.bump_basis / shell_weights)
    s = p.max() / nb
    c = (np.arange(nb) + 0.5) * s
    B = np.exp(-((p[None, :] - c[:, None]) ** 2) / (2 * s * s))
    edges = np.linspace(0.0, p.max(), nb + 1)
    idx = np.clip(np.searchsorted(edges, p, side="right") - 1, 0, nb - 1)
    wn = np.zeros_like(p)
    for q in range(nb):
        msk = idx == q
        if msk.any():
            wn[msk] = deg[msk] / deg[msk].sum()
    amps = np.random.default_rng(cfg["seed"]).uniform(0.0, 5.0, nb)
    n0 = amps @ B
    dn = B[3].copy()  # the direction of the fourth bump amplitude
    L, dlam, dm2, ddn = dual_loss(cfg["Ns"], cfg["M"], n0, 1.0, cfg["t_final"], wn, 1.0, dn, N=cfg["N"], dt=cfg["dt"],
                                  lam=cfg["lam"], mass2=cfg["mass2"])
    out = os.path.join(HERE, cfg["name"] + ".npz")
    np.savez_compressed(out, n0=n0, w_n=wn, dn=dn, amps=amps, L=L, dL=np.array([dlam, dm2, ddn]),
                        cfg=np.array([cfg["Ns"], cfg["M"], cfg["N"], cfg["lam"], cfg["dt"], cfg["mass2"],
                                      cfg["t_final"]]))
    print(f"wrote {out} ({time.time() - t_start:.0f} s): L={L!r} dL={[dlam, dm2, ddn]!r}", flush=True)


ALL = {"small": (generate, SMALL), "c1": (generate, C1), "c2": (generate, C2), "c3_ns48": (generate, C3A),
       "c3_ns24": (generate, C3B), "c4": (generate_adjoint, C4), "c5_short": (generate, C5S)}

if __name__ == "__main__":
    names = sys.argv[1:] or list(ALL)
    for nm in names:
        fn, cfg = ALL[nm]
        fn(cfg)
