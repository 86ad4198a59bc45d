"""Parity of the CUDA path (through the C ABI) with the CPU FP64 oracle.

Tolerances: plain FP64 path 1e-10 relative (F, rho normalised by their max
over the row; n per orbit and E); mixed path 1e-5 on n and E.
"""
import numpy as np
import pytest

from kbtest_util import (ENGINE_FULL, ENGINE_OCTANT, make_gpu, make_oracle, occupation, random_symmetric_row,
                         rel)

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL_MIXED = 1e-5


def run_pair(cfg, steps, precision=0, engine=ENGINE_OCTANT, check_rows=True, tol=TOL64):
    """Evolve GPU and oracle side by side; compare every measurement and rows."""
    g = make_gpu(cfg, precision)
    o = make_oracle(cfg, engine)
    _, k2, _ = g.orbits(0)
    n = occupation(cfg, k2)
    g.init(0, n, cfg.get("init_mass", 1.0))
    o.init_occupation(n, cfg.get("init_mass", 1.0))
    worst = {"E": 0.0, "n": 0.0, "F": 0.0, "rho": 0.0}
    mg, mo = g.measure(0, 2), o.measure(2)
    worst["E"] = max(worst["E"], abs(mg["E"] - mo["E"]) / abs(mo["E"]))
    for t in range(3, 3 + steps):
        g.step(t)
        o.step(t)
        mg, mo = g.measure(0, t), o.measure(t)
        worst["E"] = max(worst["E"], abs(mg["E"] - mo["E"]) / abs(mo["E"]))
        worst["n"] = max(worst["n"], rel(mg["n"], mo["n"]))
        assert abs(mg["M2"] - mo["M2"]) <= tol * abs(mo["M2"])
        assert abs(mg["E_mem"] - mo["E_mem"]) <= tol * max(abs(mo["E"]), 1e-300)
        if check_rows and (t % 7 == 0 or t == 2 + steps):
            tmin, tmax = g.window(0)
            assert (tmin, tmax) == o.window()
            for tp in range(tmin, t + 1, max(1, (t - tmin) // 5)):
                worst["F"] = max(worst["F"], rel(g.get(0, 0, t, tp), o.F(t, tp)))
                if tp < t:
                    worst["rho"] = max(worst["rho"], rel(g.get(0, 1, t, tp), o.rho(t, tp)))
    return worst, g, o


@pytest.mark.parametrize("cfg,steps", [
    (dict(Ns=8, M=24, dt=0.1, lam=1.0, T=2.0), 20),                  # window not yet full
    (dict(Ns=8, M=6, dt=0.1, lam=4.0, T=2.0), 30),                   # ring wraps many times
    (dict(Ns=16, M=40, dt=0.1, lam=1.0, T=2.0), 60),                 # config-1 lattice, wraps
    (dict(Ns=12, M=35, dt=0.05, lam=4.0, init="tsunami", init_mass=1.2), 45),
])
def test_step_parity_fp64(cfg, steps):
    worst, _, _ = run_pair(cfg, steps)
    for k, v in worst.items():
        assert v <= TOL64, (k, v)


def test_step_parity_full_lattice_engine():
    """GPU orbit path vs the oracle's full-lattice (CPUfull) engine."""
    cfg = dict(Ns=8, M=10, dt=0.1, lam=2.0, T=2.0)
    worst, _, _ = run_pair(cfg, 16, engine=ENGINE_FULL)
    for k, v in worst.items():
        assert v <= TOL64, (k, v)


@pytest.mark.parametrize("pexp", [0, 2])
def test_lo_and_classical(pexp):
    cfg = dict(Ns=8, M=9, dt=0.1, lam=3.0, T=2.0, pexp=pexp)
    worst, _, _ = run_pair(cfg, 20)
    for k, v in worst.items():
        assert v <= TOL64, (k, v)


def test_sunset_random_rows():
    """TwoPIScalar_Tests_LambdaNLO_checkfastimplementation.jl:18-125 made deterministic:
    evolve to t=10, expand, overwrite row tmone with cubic-symmetric random values,
    compute Sigma(tmone, tp) and compare site by site."""
    for Ns in (8, 16):
        cfg = dict(Ns=Ns, M=14, dt=0.01, lam=10.0, N=8, T=2.0)
        g = make_gpu(cfg)
        o = make_oracle(cfg, ENGINE_FULL if Ns == 8 else ENGINE_OCTANT)
        _, k2, _ = g.orbits(0)
        n = occupation(cfg, k2)
        g.init(0, n, 1.0)
        o.init_occupation(n, 1.0)
        for t in range(3, 11):
            g.step(t)
            o.step(t)
        g.expand()
        o.expand()
        t = 11
        tmone = t - 1
        rng = np.random.default_rng(1234 + Ns)
        for tp in range(1, t):
            Fv, rv = random_symmetric_row(g.S[0], rng), random_symmetric_row(g.S[0], rng)
            if tp == tmone:
                rv[:] = 0.0  # rho(t,t) = 0 is structural in the GPU storage
            for h in (g, ):
                h.set(0, 0, tmone, tp, Fv)
                h.set(0, 1, tmone, tp, rv)
            o.set(0, tmone, tp, Fv)
            o.set(1, tmone, tp, rv)
        g.self_energies(tmone)
        o.self_energies(tmone)
        for tp in range(1, t):
            assert rel(g.sigma(0, 1, tp), o.sigma(1, tp)) <= 1e-12
            assert rel(g.sigma(0, 0, tp), o.sigma(0, tp)) <= 1e-12


def test_invariants_and_symmetry():
    cfg = dict(Ns=8, M=7, dt=0.1, lam=2.0, T=2.0)
    _, g, _ = run_pair(cfg, 12, check_rows=False)
    tmin, t = g.window(0)
    assert np.all(g.get(0, 1, t, t) == 0.0)
    assert np.all(g.get(0, 1, t, t - 1) == cfg["dt"])
    for a in range(tmin, t + 1):
        for b in range(tmin, a):
            assert np.array_equal(g.get(0, 0, a, b), g.get(0, 0, b, a))
            assert np.array_equal(g.get(0, 1, a, b), -g.get(0, 1, b, a))


def test_traces_match():
    cfg = dict(Ns=8, M=8, dt=0.1, lam=2.0, T=2.0)
    _, g, o = run_pair(cfg, 10, check_rows=False)
    tr = g.traces(0)
    mo = o.measure(12)
    for k in ("Fonet", "ronet", "SigF", "Sigr"):
        assert rel(tr[k], mo[k]) <= TOL64, k


def test_mixed_precision_error():
    cfg = dict(Ns=16, M=40, dt=0.05, lam=4.0, init="tsunami", init_mass=1.2)
    worst, _, _ = run_pair(cfg, 80, precision=1, check_rows=False, tol=1e-6)
    assert worst["n"] <= TOL_MIXED, worst
    assert worst["E"] <= TOL_MIXED, worst


def test_graph_steps_equal_single_steps():
    cfg = dict(Ns=8, M=9, dt=0.1, lam=2.0, T=2.0)
    a, b = make_gpu(cfg), make_gpu(cfg)
    _, k2, _ = a.orbits(0)
    n = occupation(cfg, k2)
    a.init(0, n, 1.0)
    b.init(0, n, 1.0)
    for t in range(3, 23):
        a.step(t)
    meas = b.steps(3, 20, measure_every=5)
    assert b.window(0) == a.window(0)
    assert np.array_equal(a.get(0, 0, 22, 15), b.get(0, 0, 22, 15))
    assert np.array_equal(a.get(0, 1, 22, 20), b.get(0, 1, 22, 20))
    ma = a.measure(0, 22)
    mb = b.measure(0, 22)
    assert ma["E"] == mb["E"]
    assert len(meas[0]) == 4


def test_batched_runs_equal_single_runs():
    from kb2pi import capi

    cfgs = [dict(Ns=8, M=9, dt=0.05, lam=2.0, T=1.0), dict(Ns=12, M=17, dt=0.05, lam=5.0, T=2.5),
            dict(Ns=6, M=5, dt=0.05, lam=0.7, T=0.6)]
    ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=0, device=0, flags=0, dt=c["dt"],
                        lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
    batch = capi.Handle(ps)
    singles = [make_gpu(c) for c in cfgs]
    for r, c in enumerate(cfgs):
        _, k2, _ = batch.orbits(r)
        n = occupation(c, k2)
        batch.init(r, n, 1.0)
        singles[r].init(0, n, 1.0)
    for t in range(3, 25):
        batch.step(t)
        for s in singles:
            s.step(t)
    for r, s in enumerate(singles):
        assert batch.measure(r, 24)["E"] == s.measure(0, 24)["E"]
        assert np.array_equal(batch.get(r, 0, 24, 22), s.get(0, 0, 24, 22))


def test_checkpoint_roundtrip():
    cfg = dict(Ns=8, M=9, dt=0.1, lam=2.0, T=2.0)
    g = make_gpu(cfg)
    _, k2, _ = g.orbits(0)
    g.init(0, occupation(cfg, k2), 1.0)
    for t in range(3, 12):
        g.step(t)
    buf = g.checkpoint()
    for t in range(12, 17):
        g.step(t)
    e1 = g.measure(0, 16)["E"]
    row1 = g.get(0, 0, 16, 10)
    g.restore(buf)
    assert g.window(0)[1] == 11
    for t in range(12, 17):
        g.step(t)
    assert g.measure(0, 16)["E"] == e1
    assert np.array_equal(g.get(0, 0, 16, 10), row1)


def test_bad_checkpoints_are_refused():
    """Host-side faults on the checkpoint path: a buffer that is too small, one whose
    header was damaged, and one taken from a handle of another shape are refused
    with KB_ERR_PARAM before anything is copied; the handle then evolves on as if
    nothing had happened."""
    from kb2pi import capi

    cfg = dict(Ns=8, M=9, dt=0.1, lam=2.0, T=2.0)
    g = make_gpu(cfg)
    _, k2, _ = g.orbits(0)
    g.init(0, occupation(cfg, k2), 1.0)
    for t in range(3, 12):
        g.step(t)
    good = g.checkpoint()
    other = make_gpu(dict(cfg, M=10))
    other.init(0, occupation(cfg, k2), 1.0)
    for t in range(3, 6):
        other.step(t)
    wrong_shape = other.checkpoint()
    other.close()
    damaged = good.copy()
    damaged[:8] ^= 0xFF
    for buf in (good[:-64].copy(), damaged, wrong_shape):
        with pytest.raises(capi.KbError) as ei:
            g.restore(buf)
        assert ei.value.code == -1
    ref = make_gpu(cfg)
    ref.init(0, occupation(cfg, k2), 1.0)
    for t in range(3, 16):
        ref.step(t)
    for t in range(12, 16):
        g.step(t)
    assert g.measure(0, 15)["E"] == ref.measure(0, 15)["E"]
    g.close()
    ref.close()


def test_errors_are_reported():
    from kb2pi import capi

    cfg = dict(Ns=8, M=9, dt=0.1, lam=2.0, T=2.0)
    g = make_gpu(cfg)
    with pytest.raises(capi.KbError):
        g.step(3)  # before init
    _, k2, _ = g.orbits(0)
    g.init(0, occupation(cfg, k2), 1.0)
    with pytest.raises(capi.KbError):
        g.step(5)  # not lastEvolStep + 1
    for t in range(3, 14):
        g.step(t)
    with pytest.raises(capi.KbError) as ei:
        g.get(0, 0, 13, 2)  # outside the window [5, 13]
    assert ei.value.code == -6
    with pytest.raises(capi.KbError):
        make_gpu(dict(Ns=7, M=9, dt=0.1, lam=1.0))


@pytest.mark.parametrize("name", ["small_ns8_m10", "c1_ns16_m202"])
def test_gpu_matches_golden(name):
    """Committed oracle trajectories (tests/golden/make_golden.py), config 1 included."""
    import os

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz"))
    Ns, M, N, lam, dt, T, steps = g["cfg"]
    cfg = dict(Ns=int(Ns), M=int(M), N=int(N), lam=float(lam), dt=float(dt))
    h = make_gpu(cfg)
    h.init(0, g["n0"], 1.0)
    scal = [[h.measure(0, 2)[k] for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")]]
    snaps = []
    for t in range(3, 3 + int(steps)):
        h.step(t)
        m = h.measure(0, t)
        scal.append([m[k] for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")])
        if t in set(g["n_t"].tolist()):
            snaps.append(m["n"])
    scal = np.array(scal)
    ref = g["scalars"]
    for col in range(1, 6):
        assert rel(scal[:, col], ref[:, col]) <= TOL64, col
    assert rel(np.array(snaps), g["n"]) <= TOL64
    t = 2 + int(steps)
    for i, tp in enumerate(g["tps"]):
        assert rel(h.get(0, 0, t, int(tp)), g["F_last_row"][i]) <= TOL64
        if tp < t:
            assert rel(h.get(0, 1, t, int(tp)), g["rho_last_row"][i]) <= TOL64


def test_gauss_zero_plus_one_dimensions():
    """Nx = 1 Gauss state (Simulationfiles/Anders_NNLOpaper.jl parameters) on the GPU:
    E(2) is the reference's analytic energy and the run follows the oracle."""
    from oracle import Oracle

    xi, eta, sig, lam, N, dt = 0.4, 5.0, 1.0, 1.0, 8, 0.01
    E0 = 0.5 * eta ** 2 + sig ** 2 / (8 * xi ** 2) + 0.5 * xi ** 2 + (1 / 24) * lam * (N + 2) / N * xi ** 4
    h = make_gpu(dict(Ns=1, M=300, N=N, lam=lam, dt=dt))
    F11 = np.array([xi ** 2])
    F21 = xi * eta * dt + F11
    F22 = (eta ** 2 + sig ** 2 / (4 * xi ** 2)) * dt ** 2 - F11 + 2 * F21
    h.init_rows(0, F11, F21, F22)
    o = Oracle(1, 3, M=300, N=N, dt=dt, lam=lam, mass2=1.0, engine=ENGINE_FULL)
    o.init_gauss(xi, eta, sig)
    assert abs(h.measure(0, 2)["E"] - E0) <= 1e-12 * E0
    for t in range(3, 400):
        h.step(t)
        o.step(t)
    mg, mo = h.measure(0, 399), o.measure(399)
    assert abs(mg["E"] - mo["E"]) <= TOL64 * abs(mo["E"])


def test_host_mirror_run_simulation():
    """The reference's driver loop (G_SimulationArgs.jl:86-106) through kb2pi's mirror
    of QFTdynamicsProblem / initialize! / evolve! / measure!, against the oracle."""
    import kb2pi
    from oracle import Oracle

    parameters = {"Mass": 1.0, "Nx": 8, "sdim": 3, "dt": 0.1, "Nsteps": 20, "NstepsinMemory": 12, "Nmeas": 0,
                  "Mod": "phi4", "Lambda": 2.0, "ONgroup": 4, "init": "Thermal", "T": 2.0, "Reno": "RMass",
                  "Pexp": "LambdaNLO", "Num": "GPU", "Nchunks": 0, "tag": "test", "ov": True}
    sol = kb2pi.run_simulation(dict(parameters))
    problem = sol.problem
    o = Oracle(8, 3, M=12, N=4, dt=0.1, lam=2.0, mass2=problem.model.Mass2, mass=1.0)
    _, k2, _ = o.orbits()
    o.init_occupation(1.0 / (np.exp(np.sqrt(k2 + 1.0) / 2.0) - 1.0), 1.0)
    Es = [o.measure(2)["E"]]
    for t in range(3, 23):
        o.step(t)
        Es.append(o.measure(t)["E"])
    got = [m["E"] for m in sol.measurearray]
    assert len(got) == 21
    assert rel(got, Es) <= TOL64
    assert problem.model.Mass2 < 1.0  # RMass counterterm applied


@pytest.mark.parametrize("num", ["GPU", "GPUmixed"])
def test_host_mirror_tachyonic(num):
    """Phi4Tachyonic with RMass (TwoPIScalar_ModelExpansionRenormalization.jl:11-16, 30-36):
    the bare m^2 = -Mass^2 + counterterm is negative and initialize! uses disc.Mass
    (TwoPIScalar_Initialization.jl:295); the GPU run follows the oracle evolved with that
    negative m^2 (1e-10 FP64, 1e-5 mixed) in E, M^2 and n."""
    import kb2pi
    from oracle import Oracle

    parameters = {"Mass": 1.0, "Nx": 10, "sdim": 3, "dt": 0.1, "Nsteps": 30, "NstepsinMemory": 14, "Nmeas": 0,
                  "Mod": "phi4tachyonic", "Lambda": 3.0, "ONgroup": 4, "init": "Thermal", "T": 1.5,
                  "Reno": "RMass", "Pexp": "LambdaNLO", "Num": num}
    sol = kb2pi.run_simulation(dict(parameters))
    problem = sol.problem
    assert problem.model.tachyonic and problem.model.Mass2 < -1.0
    o = Oracle(10, 3, M=14, N=4, dt=0.1, lam=3.0, mass2=problem.model.Mass2, mass=1.0)
    _, k2, _ = o.orbits()
    o.init_occupation(1.0 / (np.exp(np.sqrt(k2 + 1.0) / 1.5) - 1.0), 1.0)
    ref = [o.measure(2)]
    for t in range(3, 33):
        o.step(t)
        ref.append(o.measure(t))
    tol = TOL64 if num == "GPU" else TOL_MIXED
    got = sol.measurearray
    assert len(got) == 31
    assert rel([m["E"] for m in got], [m["E"] for m in ref]) <= tol
    assert rel([m["M2"] for m in got], [m["M2"] for m in ref]) <= tol
    assert max(m["M2"] for m in ref) < 0.0  # the effective mass stays negative: unstable low modes
    for mg, mo in zip(got[1:], ref[1:]):
        assert rel(mg["n"], mo["n"]) <= tol


@pytest.mark.parametrize("pexp_name,pexp", [("NinverseNLO", 4), ("NinverseLO", 3)])
def test_host_mirror_ninverse(pexp_name, pexp):
    """The driver loop with Pexp = NinverseNLO / NinverseLO and RMass renormalisation
    (its counterterm uses the 1/N Hartree prefactor), against the oracle."""
    import kb2pi
    from oracle import Oracle

    parameters = {"Mass": 1.0, "Nx": 6, "sdim": 3, "dt": 0.1, "Nsteps": 16, "NstepsinMemory": 9, "Nmeas": 0,
                  "Mod": "phi4", "Lambda": 3.0, "ONgroup": 4, "init": "Thermal", "T": 1.5, "Reno": "RMass",
                  "Pexp": pexp_name, "Num": "GPU"}
    sol = kb2pi.run_simulation(dict(parameters))
    problem = sol.problem
    o = Oracle(6, 3, M=9, N=4, dt=0.1, lam=3.0, mass2=problem.model.Mass2, mass=1.0, pexp=pexp)
    _, k2, _ = o.orbits()
    o.init_occupation(1.0 / (np.exp(np.sqrt(k2 + 1.0) / 1.5) - 1.0), 1.0)
    Es = [o.measure(2)["E"]]
    for t in range(3, 19):
        o.step(t)
        Es.append(o.measure(t)["E"])
    assert rel([m["E"] for m in sol.measurearray], Es) <= TOL64
    assert problem.model.Mass2 < 1.0


def c3_runs(nruns, seed, Ns_choices, M_range):
    """Config 3 style batch: per-run seeded draws of Ns, lambda, T and the memory window."""
    rng = np.random.default_rng(seed)
    runs = []
    for r in range(nruns):
        runs.append(dict(Ns=int(rng.choice(Ns_choices)), lam=float(rng.uniform(0.5, 8.0)),
                         T=float(rng.uniform(0.5, 3.0)), M=int(rng.integers(M_range[0], M_range[1] + 1)),
                         dt=0.05, N=4))
    return runs


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_config3_style(precision):
    """Uneven runs in one launch per kernel: each run of the batch is bit-identical to
    the same run alone, and follows the FP64 oracle (1e-10 plain, 1e-5 mixed)."""
    from kb2pi import capi

    runs = c3_runs(12, 2024, [6, 8, 12, 16], (8, 40))
    ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=precision, device=0, flags=0,
                        dt=c["dt"], lam=c["lam"], mass2=1.0, mass=1.0) for c in runs]
    batch = capi.Handle(ps)
    alone = [make_gpu(c, precision) for c in runs[:3]]
    oracles = [make_oracle(c) for c in runs]
    for r, c in enumerate(runs):
        _, k2, _ = batch.orbits(r)
        n = occupation(c, k2)
        batch.init(r, n, 1.0)
        oracles[r].init_occupation(n, 1.0)
        if r < 3:
            alone[r].init(0, n, 1.0)
    steps = 50
    batch.steps(3, steps, 0)
    for a in alone:
        a.steps(3, steps, 0)
    for o in oracles:
        for t in range(3, 3 + steps):
            o.step(t)
    t = 2 + steps
    tol = TOL64 if precision == 0 else TOL_MIXED
    for r in range(len(runs)):
        mb, mo = batch.measure(r, t), oracles[r].measure(t)
        assert abs(mb["E"] - mo["E"]) <= tol * abs(mo["E"]), r
        assert rel(mb["n"], mo["n"]) <= tol, r
        if r < 3:
            assert mb["E"] == alone[r].measure(0, t)["E"]
            assert np.array_equal(mb["n"], alone[r].measure(0, t)["n"])


@pytest.mark.parametrize("precision", [0, 1])
def test_device_measurement_stream(precision, tmp_path):
    """kb_steps_recorded: the measurements recorded on the device inside the step
    graph equal kb_measure after single steps, bitwise; the host mirror's
    stream path fills the same measurearray, which round-trips through save/load."""
    import kb2pi

    cfg = dict(Ns=10, M=30, N=4, lam=3.0, dt=0.1, pexp=1, T=1.5)
    a = make_gpu(cfg, precision)
    b = make_gpu(cfg, precision)
    _, k2, _ = a.orbits()
    n0 = occupation(cfg, k2)
    a.init(0, n0, 1.0)
    b.init(0, n0, 1.0)
    every = 7
    rec = a.steps_recorded(3, 50, every)
    ref = []
    for t in range(3, 53):
        b.step(t)
        if (t - 2) % every == 0:
            ref.append((t, b.measure(0, t)))
    assert len(rec) == len(ref) == 7
    for row, (t, m) in zip(rec, ref):
        d = row[0]
        assert d["t"] == t
        for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2"):
            assert d[k] == m[k], k
        for k in ("F", "ddF", "n", "omega", "c"):
            assert np.array_equal(d[k], m[k]), k
    a.close()
    b.close()
    params = {"Mass": 1.0, "Nx": 10, "sdim": 3, "dt": 0.1, "Nsteps": 60, "NstepsinMemory": 30, "Nmeas": 6,
              "Mod": "phi4", "Lambda": 3.0, "ONgroup": 4, "init": "Thermal", "T": 1.5, "Reno": "RNone",
              "Pexp": "LambdaNLO", "Num": "GPU" if precision == 0 else "GPUmixed"}
    s1 = kb2pi.run_simulation(params)
    s2 = kb2pi.run_simulation(params, stream=True)
    for m1, m2 in zip(s1.measurearray, s2.measurearray):
        assert m1["E"] == m2["E"] and np.array_equal(m1["n"], m2["n"])
    path = str(tmp_path / "Measurearray.npz")
    assert kb2pi.save_measurearray(path, s2, params) == 7
    back, p2 = kb2pi.load_measurearray(path)
    assert p2 == params and len(back) == 7
    for m1, m2 in zip(s2.measurearray, back):
        assert m1["E"] == m2["E"] and np.array_equal(m1["n"], m2["n"])


@pytest.mark.parametrize("precision", [0, 1])
def test_pipelined_measurement(precision):
    """kb_measure_enqueue / kb_measure_take with the next step issued before the
    take equal kb_measure after each step, bitwise; a take of a step that was
    not queued (or was taken already) and an enqueue of an old step fail."""
    from kb2pi import capi

    cfg = dict(Ns=10, M=12, N=4, lam=3.0, dt=0.1, pexp=1, T=1.5)
    a = make_gpu(cfg, precision)
    b = make_gpu(cfg, precision)
    _, k2, _ = a.orbits()
    n0 = occupation(cfg, k2)
    a.init(0, n0, 1.0)
    b.init(0, n0, 1.0)
    ref, got = {}, {}
    a.step(3)
    a.measure_enqueue(0, 3)
    for t in range(3, 30):
        b.step(t)
        ref[t] = b.measure(0, t)
        if t + 1 < 30:
            a.step(t + 1)
            a.measure_enqueue(0, t + 1)
        got[t] = a.measure_take(0, t)
    for t in ref:
        for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2"):
            assert got[t][k] == ref[t][k], (t, k)
        for k in ("F", "ddF", "n", "omega", "c"):
            assert np.array_equal(got[t][k], ref[t][k]), (t, k)
    with pytest.raises(capi.KbError):
        a.measure_take(0, 29)  # taken already
    with pytest.raises(capi.KbError):
        a.measure_enqueue(0, 28)  # not the last evolved step
    a.close()
    b.close()


# --- 1/N expansion (NinverseLO, NinverseNLO) -----------------------------------

@pytest.mark.parametrize("cfg,steps", [
    (dict(Ns=6, M=8, dt=0.1, lam=4.0, T=2.0, pexp=4), 24),            # ring wraps
    (dict(Ns=8, M=20, dt=0.1, lam=2.0, T=1.5, pexp=4), 30),
    (dict(Ns=12, M=14, dt=0.05, lam=3.0, init="tsunami", init_mass=1.2, pexp=4), 20),
    (dict(Ns=8, M=9, dt=0.1, lam=3.0, T=2.0, pexp=3), 20),            # NinverseLO: tadpole lambda/6
])
def test_ninverse_parity_fp64(cfg, steps):
    worst, _, _ = run_pair(cfg, steps)
    for k, v in worst.items():
        assert v <= TOL64, (k, v)


def test_ninverse_full_lattice_engine():
    """GPU bubbles + Volterra solves vs the literal full-lattice restatement of
    calcIrs!/calcIFs!/calcSelfEnergyattp! (CPUfull)."""
    cfg = dict(Ns=4, M=6, dt=0.1, lam=4.0, T=2.0, pexp=4)
    worst, _, _ = run_pair(cfg, 14, engine=ENGINE_FULL)
    for k, v in worst.items():
        assert v <= TOL64, (k, v)


def test_ninverse_batched_with_lambda_runs_and_checkpoint():
    """One FP64 handle holding a LambdaNLO run and two NinverseNLO runs equals the
    single-run handles bitwise; a checkpoint restores the bubble rings too."""
    from kb2pi import capi

    cfgs = [dict(Ns=6, M=8, lam=2.0, pexp=1, T=1.5), dict(Ns=8, M=11, lam=3.0, pexp=4, T=2.0),
            dict(Ns=6, M=7, lam=1.5, pexp=4, T=1.0)]

    def params(c):
        return capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=c["pexp"], precision=0, device=0, flags=0,
                             dt=0.1, lam=c["lam"], mass2=1.0, mass=1.0)

    hb = capi.Handle([params(c) for c in cfgs])
    singles = [capi.Handle([params(c)]) for c in cfgs]
    for r, c in enumerate(cfgs):
        _, k2, _ = hb.orbits(r)
        n = occupation(c, k2)
        hb.init(r, n, 1.0)
        singles[r].init(0, n, 1.0)
    for t in range(3, 15):
        hb.step(t)
        for s in singles:
            s.step(t)
    buf = hb.checkpoint()
    for t in range(15, 25):
        hb.step(t)
        for s in singles:
            s.step(t)
    for r, s in enumerate(singles):
        a, b = hb.measure(r, 24), s.measure(0, 24)
        assert a["E"] == b["E"] and np.array_equal(a["n"], b["n"])
    e_before = [hb.measure(r, 24)["E"] for r in range(3)]
    hb.restore(buf)
    for t in range(15, 25):
        hb.step(t)
    assert [hb.measure(r, 24)["E"] for r in range(3)] == e_before
    for h in [hb] + singles:
        h.close()


def test_ninverse_mixed_precision_is_rejected():
    from kb2pi import capi

    with pytest.raises(capi.KbError, match="1/N"):
        make_gpu(dict(Ns=6, M=8, dt=0.1, lam=2.0, pexp=4), precision=1)


@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_one_run_stays_in_that_run(precision):
    """Host-side fault injection: a NaN in one run's initial occupation surfaces as
    KB_ERR_NAN from that run's measurement alone; the other runs of the batch are
    bitwise those of the same batch without the NaN."""
    from kb2pi import capi

    runs = [dict(Ns=8, M=9, lam=2.0, T=1.5), dict(Ns=6, M=7, lam=3.0, T=2.0), dict(Ns=8, M=12, lam=1.5, T=1.0)]

    def batch(poison):
        ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=precision, device=0, flags=0,
                            dt=0.1, lam=c["lam"], mass2=1.0, mass=1.0) for c in runs]
        h = capi.Handle(ps)
        for r, c in enumerate(runs):
            _, k2, _ = h.orbits(r)
            n = occupation(c, k2)
            if poison and r == 1:
                n[3] = np.nan
            h.init(r, n, 1.0)
        h.steps(3, 16, 0)
        return h

    clean, bad = batch(False), batch(True)
    t = 18
    with pytest.raises(capi.KbError) as ei:
        bad.measure(1, t)
    assert ei.value.code == -4  # KB_ERR_NAN
    for r in (0, 2):
        a, b = clean.measure(r, t), bad.measure(r, t)
        assert a["E"] == b["E"] and np.array_equal(a["n"], b["n"])
        assert np.array_equal(clean.get(r, 0, t, t - 3), bad.get(r, 0, t, t - 3))
    clean.close()
    bad.close()
