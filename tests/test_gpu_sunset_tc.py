"""The tensor-core sunset (sunset_variant 2, tcgen05.mma kind::tf32 with each FP32
operand split into a TF32 head and tail) against the CPU FP64 oracle.

Tolerances: the mixed-precision bound, 1e-5 relative (each Sigma row normalised by
its max), for the transforms on random cubic-symmetric rows and for whole runs.
"""
import os

import numpy as np
import pytest

from kbtest_util import make_gpu, make_oracle, occupation, random_symmetric_row, rel

pytestmark = pytest.mark.gpu

TOL = 1e-5


def sigma_rows(Ns, variant, seed=7):
    """Sigma(t-1, t') of random cubic-symmetric rows on the GPU (mixed precision,
    the given sunset variant) and in the oracle."""
    cfg = dict(Ns=Ns, M=14, dt=0.01, lam=10.0, N=8, T=2.0)
    g = make_gpu(cfg, 1)
    g.set_tuning(sunset_variant=variant)
    o = make_oracle(cfg)
    _, k2, _ = g.orbits(0)
    n = occupation(cfg, k2)
    g.init(0, n, 1.0)
    o.init_occupation(n, 1.0)
    for t in range(3, 11):
        g.step(t)
        o.step(t)
    g.expand()
    o.expand()
    tmone = 10
    rng = np.random.default_rng(seed + Ns)
    for tp in range(1, tmone + 1):
        Fv, rv = random_symmetric_row(g.S[0], rng), random_symmetric_row(g.S[0], rng)
        if tp == tmone:
            rv[:] = 0.0
        g.set(0, 0, tmone, tp, Fv)
        g.set(0, 1, tmone, tp, rv)
        o.set(0, tmone, tp, Fv)
        o.set(1, tmone, tp, rv)
    g.self_energies(tmone)
    o.self_energies(tmone)
    out = [(g.sigma(0, 0, tp), g.sigma(0, 1, tp), o.sigma(0, tp), o.sigma(1, tp)) for tp in range(1, tmone + 1)]
    g.close()
    o.close()
    return out


@pytest.mark.parametrize("Ns", [2, 4, 8, 12, 16, 24, 32, 48, 64])
def test_tensor_core_sunset_matches_oracle(Ns):
    worst = 0.0
    for gF, gr, oF, orr in sigma_rows(Ns, 2):
        worst = max(worst, rel(gF, oF), rel(gr, orr))
    print(f"\ntensor-core sunset Ns={Ns}: max rel err vs FP64 oracle {worst:.2e}")
    assert worst <= TOL


def test_tensor_core_sunset_matches_cuda_core_sunset():
    a = sigma_rows(24, 2)
    b = sigma_rows(24, 0)
    for (aF, ar, _, _), (bF, br, _, _) in zip(a, b):
        assert rel(aF, bF) <= TOL and rel(ar, br) <= TOL


def test_tensor_core_sunset_config2_run():
    """Config 2 (Ns=32, M=400, 1000 steps) with the tensor-core sunset against the
    oracle trajectory: n, E and the last F, rho rows within 1e-5."""
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c2_ns32_m400.npz"))
    Ns, M, N, lam, dt, _, steps = g["cfg"]
    h = make_gpu(dict(Ns=int(Ns), M=int(M), N=int(N), lam=float(lam), dt=float(dt)), 1)
    h.set_tuning(sunset_variant=2)
    h.init(0, g["n0"], float(g["init_mass"]))
    Es, ns = [], []
    t = 2
    while t < 2 + int(steps):
        meas = h.steps(t + 1, 50, 1)
        Es.extend(d["E"] for d in meas[0])
        t += 50
        ns.append(h.measure(0, t)["n"])
    errs = {"E": rel(Es, g["scalars"][1:, 1]), "n": rel(np.array(ns), g["n"])}
    errs["F"] = max(rel(h.get(0, 0, t, int(tp)), g["F_last_row"][i]) for i, tp in enumerate(g["tps"]))
    errs["rho"] = max(rel(h.get(0, 1, t, int(tp)), g["rho_last_row"][i]) for i, tp in enumerate(g["tps"]) if tp < t)
    h.close()
    print("\nconfig 2 mixed, tensor-core sunset vs oracle: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    for k, v in errs.items():
        assert v <= TOL, (k, v)


def test_tensor_core_sunset_batch_of_uneven_runs():
    """Runs of several lattices in one launch (the kernel rebuilds its tables when
    the run changes) follow the oracle, and each equals the same run alone, bitwise."""
    from kb2pi import capi

    cfgs = [dict(Ns=24, M=30, lam=2.0, T=1.0), dict(Ns=8, M=41, lam=4.0, T=2.0), dict(Ns=16, M=37, lam=1.0, T=0.7),
            dict(Ns=6, M=9, lam=3.0, T=1.5)]
    ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=1, device=0, flags=0, dt=0.1,
                        lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
    h = capi.Handle(ps)
    h.set_tuning(sunset_variant=2)
    oracles = []
    for r, c in enumerate(cfgs):
        _, k2, _ = h.orbits(r)
        n = occupation(dict(c), k2)
        h.init(r, n, 1.0)
        o = make_oracle(dict(c, dt=0.1))
        o.init_occupation(n, 1.0)
        oracles.append(o)
    h.steps(3, 40, 0)
    for o in oracles:
        for t in range(3, 43):
            o.step(t)
    for r, c in enumerate(cfgs):
        mb, mo = h.measure(r, 42), oracles[r].measure(42)
        assert abs(mb["E"] - mo["E"]) <= TOL * abs(mo["E"]), r
        assert rel(mb["n"], mo["n"]) <= TOL, r
        a = make_gpu(dict(c, dt=0.1), 1)
        a.set_tuning(sunset_variant=2)
        _, k2, _ = a.orbits()
        a.init(0, occupation(dict(c), k2), 1.0)
        a.steps(3, 40, 0)
        ma = a.measure(0, 42)
        a.close()
        assert ma["E"] == mb["E"] and np.array_equal(ma["n"], mb["n"]), r
    h.close()
