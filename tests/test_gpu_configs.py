"""Parity at the stated sizes of the benchmark configurations, against committed
oracle trajectories (tests/golden/make_golden.py):

  config 2  Ns=32, N=4, lambda=4, dt=0.05, M=400, 1000 steps, tsunami state with
            the gap-mass initialisation (TwoPIScalar_Initialization.jl:309-314)
  config 3  the 64-run batch (Ns from {16,24,32,48}, lambda U[0.5,8], T U[0.5,3],
            M U{100..500}, dt=0.05, 500 steps, seed 12345) in one handle; its
            first Ns=48 run (M=442) and first Ns=24 run (M=164) are compared
  Ns=64     the headline lattice (config 5's Ns, N, lambda, dt and initial state) on a
            128-step window, 200 steps
  config 4  kb_adjoint at Ns=24, M=300, 300 steps, checkpoint every 20, against
            forward-mode dual numbers through the oracle (orc_dual_loss)

Tolerances: plain FP64 1e-10 relative in E, E_pot, E_kin, E_mem, M^2 (every step),
n per orbit (every 50 steps) and the sampled F, rho rows at the last time (each
normalised by its max over the trajectory or row); mixed precision 1e-5 on n and
E, with the F, rho row errors checked at the same bound. The mixed errors are
printed (pytest -s) next to the bound.
"""
import os

import numpy as np
import pytest

from kbtest_util import make_gpu, rel

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL64 = 1e-10
TOL_MIXED = 1e-5
SCAL = ("time", "E", "E_pot", "E_kin", "E_mem", "M2")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def c3_draw(seed=12345, nruns=64):
    """The config-3 batch in the order of the benchmark's draw (bench.py run_batched)."""
    rng = np.random.default_rng(seed)
    runs = []
    for _ in range(nruns):
        runs.append(dict(Ns=int(rng.choice([16, 24, 32, 48])), lam=float(rng.uniform(0.5, 8.0)),
                         T=float(rng.uniform(0.5, 3.0)), M=int(rng.integers(100, 501))))
    return runs


def evolve_recording(h, runs, steps, n_every):
    """Steps 3 .. 2 + steps in graph blocks of n_every, the scalars of every step
    (kb_steps, measure_every = 1) and n of every run at each block end."""
    scal = {r: [[h.measure(r, 2, arrays=False)[k] for k in SCAL]] for r in runs}
    nsnap = {r: [] for r in runs}
    t = 2
    while t < 2 + steps:
        cnt = min(n_every, 2 + steps - t)
        meas = h.steps(t + 1, cnt, 1)
        for r in runs:
            scal[r].extend([[d[k] for k in SCAL] for d in meas[r]])
        t += cnt
        for r in runs:
            nsnap[r].append(h.measure(r, t)["n"])
    return {r: np.array(v) for r, v in scal.items()}, {r: np.array(v) for r, v in nsnap.items()}, t


def compare(h, run, g, scal, nsnap, t, tol):
    """Worst relative errors of one run against its fixture (and asserts them)."""
    worst = {}
    for col, k in enumerate(SCAL[1:], start=1):
        worst[k] = rel(scal[:, col], g["scalars"][:, col])
    worst["n"] = rel(nsnap, g["n"])
    assert scal.shape == g["scalars"].shape and nsnap.shape == g["n"].shape
    wF, wr = 0.0, 0.0
    for i, tp in enumerate(g["tps"]):
        wF = max(wF, rel(h.get(run, 0, t, int(tp)), g["F_last_row"][i]))
        if tp < t:
            wr = max(wr, rel(h.get(run, 1, t, int(tp)), g["rho_last_row"][i]))
    worst["F"], worst["rho"] = wF, wr
    return worst


@pytest.mark.parametrize("precision,compensated", [(0, 0), (1, 0), (1, 1)])
def test_config2_full_size(precision, compensated):
    """compensated = 1: the mixed path with Kahan-compensated FP32 tile sums."""
    g = load("c2_ns32_m400")
    Ns, M, N, lam, dt, _, steps = g["cfg"]
    cfg = dict(Ns=int(Ns), M=int(M), N=int(N), lam=float(lam), dt=float(dt))
    h = make_gpu(cfg, precision)
    if compensated:
        h.set_tuning(memint_variant=2, memint_compensated=1)
        assert h.tuning()["memint_compensated"] == 1
    h.init(0, g["n0"], float(g["init_mass"]))
    scal, nsnap, t = evolve_recording(h, [0], int(steps), 50)
    assert t == 1002 and np.array_equal(g["n_t"], np.arange(52, 1003, 50))
    worst = compare(h, 0, g, scal[0], nsnap[0], t, TOL64)
    h.close()
    print(f"\nconfig 2 {'FP64' if precision == 0 else 'mixed'}{' compensated' if compensated else ''} vs oracle: " +
          ", ".join(f"{k} {v:.2e}" for k, v in worst.items()))
    if precision == 0:
        for k, v in worst.items():
            assert v <= TOL64, (k, v)
    else:
        for k in ("n", "E", "F", "rho"):
            assert worst[k] <= TOL_MIXED, (k, worst[k])


@pytest.mark.parametrize("precision", [0, 1])
def test_config3_full_batch(precision):
    """All 64 runs in one handle for 500 steps; the runs with fixtures follow the oracle."""
    from kb2pi import capi

    runs = c3_draw()
    fixtures = {}
    for name in ("c3_ns48_m442", "c3_ns24_m164"):
        g = load(name)
        r = int(g["batch_index"])
        c = runs[r]
        assert (c["Ns"], c["M"]) == (int(g["cfg"][0]), int(g["cfg"][1])) and c["lam"] == float(g["cfg"][3])
        fixtures[r] = g
    ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=precision, device=0, flags=0, dt=0.05,
                        lam=c["lam"], mass2=1.0, mass=1.0) for c in runs]
    h = capi.Handle(ps)
    for r, c in enumerate(runs):
        _, k2, _ = h.orbits(r)
        n = 1.0 / (np.exp(np.sqrt(k2 + 1.0) / c["T"]) - 1.0)
        if r in fixtures:
            assert rel(n, fixtures[r]["n0"]) <= 1e-15
        h.init(r, n, 1.0)
    scal, nsnap, t = evolve_recording(h, sorted(fixtures), 500, 50)
    assert t == 502
    for r, g in fixtures.items():
        assert h.window(r) == (max(1, 502 - runs[r]["M"] + 1), 502)  # the window wrapped
        worst = compare(h, r, g, scal[r], nsnap[r], t, TOL64)
        print(f"\nconfig 3 run {r} (Ns={runs[r]['Ns']}, M={runs[r]['M']}) "
              f"{'FP64' if precision == 0 else 'mixed'} vs oracle: " +
              ", ".join(f"{k} {v:.2e}" for k, v in worst.items()))
        if precision == 0:
            for k, v in worst.items():
                assert v <= TOL64, (r, k, v)
        else:
            for k in ("n", "E", "F", "rho"):
                assert worst[k] <= TOL_MIXED, (r, k, worst[k])
    h.close()


@pytest.mark.parametrize("precision,sunset_variant", [(0, 0), (1, 0), (1, 2)])
def test_headline_lattice_ns64(precision, sunset_variant):
    """The headline lattice (Ns=64, N=4, lambda=2, dt=0.05, tsunami state with the gap
    mass) on a 128-step window for 200 steps, so the window wraps; sunset_variant 2 is
    the tensor-core sunset."""
    g = load("c5_ns64_m128")
    Ns, M, N, lam, dt, _, steps = g["cfg"]
    h = make_gpu(dict(Ns=int(Ns), M=int(M), N=int(N), lam=float(lam), dt=float(dt)), precision)
    h.set_tuning(sunset_variant=sunset_variant)
    h.init(0, g["n0"], float(g["init_mass"]))
    scal, nsnap, t = evolve_recording(h, [0], int(steps), 50)
    assert t == 202 and h.window(0) == (202 - int(M) + 1, 202)
    worst = compare(h, 0, g, scal[0], nsnap[0], t, TOL64)
    h.close()
    print(f"\nNs=64 {'FP64' if precision == 0 else 'mixed'} sunset variant {sunset_variant} vs oracle: " +
          ", ".join(f"{k} {v:.2e}" for k, v in worst.items()))
    if precision == 0:
        for k, v in worst.items():
            assert v <= TOL64, (k, v)
    else:
        for k in ("n", "E", "F", "rho"):
            assert worst[k] <= TOL_MIXED, (k, worst[k])


def test_config4_adjoint_matches_dual_numbers():
    """Exact derivatives on both sides at the config-4 size: d/dlambda, d/dm^2 and
    the derivative along the fourth bump of the initial occupation."""
    from kb2pi import adjoint as adj

    g = load("c4_adjoint_ns24_m300")
    Ns, M, N, lam, dt, mass2, tf = g["cfg"]
    cfg = dict(Ns=int(Ns), M=int(M), N=int(N), lam=float(lam), dt=float(dt), mass2=float(mass2))
    hh = make_gpu(cfg)
    _, k2, deg = hh.orbits(0)
    hh.close()
    B = adj.bump_basis(k2, 8)
    assert rel(g["amps"] @ B, g["n0"]) <= 1e-15
    assert rel(adj.shell_weights(k2, deg, 8), g["w_n"]) <= 1e-15
    r = adj.loss_and_grad(cfg, g["n0"], int(tf), w_n=g["w_n"], w_E=1.0, ckpt_every=20)
    L = float(g["L"])
    dlam, dm2, ddn = g["dL"]
    errs = {"loss": abs(r["loss"] - L) / abs(L), "lambda": abs(r["lambda"] - dlam) / abs(dlam),
            "mass2": abs(r["mass2"] - dm2) / abs(dm2),
            "occupation": abs(float(np.dot(r["n_init"], g["dn"])) - ddn) / abs(ddn)}
    print("\nconfig 4 adjoint vs dual numbers: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert errs["loss"] <= 1e-10
    for k in ("lambda", "mass2", "occupation"):
        assert errs[k] <= 1e-6, (k, errs[k])
