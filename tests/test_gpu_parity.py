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
