"""The CPU FP64 oracle, pinned before the CUDA path is compared against it.

The Julia reference cannot run here, so the oracle is pinned against
independent implementations and known answers: numpy's pocketfft for the
sunset (the rfft/brfft convention of TwoPIScalar_Evolution.jl:25-31), the
closed-form lambda = 0 solution, the reference's analytic Gauss energy
(TwoPIScalar_Initialization.jl:109) and agreement of its three engines.
"""
import os

import numpy as np
import pytest

from oracle import ENGINE_FULL, ENGINE_OCTANT, ENGINE_ORBIT, PEXP_LO, PEXP_NLO_CLASSICAL, Oracle
from kbtest_util import make_oracle, thermal_n

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def numpy_sunset(Fl, rl, lam, N, classical=False):
    """Line-by-line numpy restatement of calcSelfEnergyattpsimple!
    (TwoPIScalar_Evolution.jl:130-139): real(rfft), pointwise, brfft."""
    V = Fl.size
    iv = 1.0 / V
    axes = tuple(range(Fl.ndim))
    rx = np.real(np.fft.rfftn(rl, axes=axes))
    Fx = np.real(np.fft.rfftn(Fl, axes=axes))
    if classical:
        Sr, SF = rx * Fx ** 2, Fx * Fx ** 2
    else:
        Sr, SF = rx * (Fx ** 2 - (1 / 12.) * rx ** 2), Fx * (Fx ** 2 - 0.75 * rx ** 2)
    brfft = lambda X: np.fft.irfftn(X, s=Fl.shape, axes=axes) * V  # noqa: E731  unnormalised backward
    sr = iv ** 3 * (-lam ** 2 * (N + 2) / (6 * N ** 2)) * brfft(Sr)
    sF = iv ** 3 * (-lam ** 2 * (N + 2) / (18 * N ** 2)) * brfft(SF)
    return sF, sr


@pytest.mark.parametrize("Ns", [4, 6, 8, 12])
@pytest.mark.parametrize("engine", [ENGINE_FULL, ENGINE_ORBIT, ENGINE_OCTANT])
def test_sunset_matches_numpy(Ns, engine):
    lam, N = 3.0, 4
    o = Oracle(Ns, 3, M=4, N=N, lam=lam, engine=engine)
    rng = np.random.default_rng(Ns)
    F = rng.random(o.S) - 0.5
    r = rng.random(o.S) - 0.5
    sF, sr = o.sunset_rows(F, r)
    so = o.site_orbit()
    shape = (Ns, Ns, Ns)
    sFn, srn = numpy_sunset(F[so].reshape(shape, order="F"), r[so].reshape(shape, order="F"), lam, N)
    sFn, srn = sFn.reshape(-1, order="F"), srn.reshape(-1, order="F")
    # every site of an orbit carries the same value (cubic symmetry is preserved)
    for k in range(o.S):
        sites = np.where(so == k)[0]
        assert np.ptp(srn[sites]) <= 1e-13 * np.max(np.abs(srn))
        assert abs(sF[k] - sFn[sites[0]]) <= 1e-13 * np.max(np.abs(sFn))
        assert abs(sr[k] - srn[sites[0]]) <= 1e-13 * np.max(np.abs(srn))


def test_orbit_tables():
    from kb2pi.twopiscalar import lattice_orbits

    for Ns in (2, 4, 8, 16, 24):
        o = Oracle(Ns, 3, M=4)
        rep, k2, deg = o.orbits()
        assert deg.sum() == Ns ** 3
        H = Ns // 2 + 1
        assert o.S == H * (H + 1) * (H + 2) // 6
        r2, k22, d2 = lattice_orbits(Ns)
        assert np.array_equal(rep, r2) and np.array_equal(deg, d2)
        assert np.allclose(k2, k22, rtol=0, atol=1e-14)
        expect = (4 * np.sin(np.pi * rep / Ns) ** 2).sum(axis=1)
        assert np.allclose(k2, expect, atol=1e-14)


def _run(engine, cfg, steps, pexp=1):
    o = Oracle(cfg["Ns"], 3, M=cfg["M"], N=4, dt=cfg["dt"], lam=cfg["lam"], engine=engine, pexp=pexp,
               nthreads=3)
    _, k2, _ = o.orbits()
    o.init_occupation(1.0 / (np.exp(np.sqrt(k2 + 1.0) / 2.0) - 1.0), 1.0)
    ms = [o.measure(2)]
    for t in range(3, 3 + steps):
        o.step(t)
        ms.append(o.measure(t))
    return o, ms


@pytest.mark.parametrize("pexp", [PEXP_LO, 1, PEXP_NLO_CLASSICAL])
def test_engines_agree(pexp):
    """CPUfull (full lattice + FFT), CPUred (orbits + FFT) and the octant form."""
    cfg = dict(Ns=6, M=7, dt=0.1, lam=4.0)
    runs = {e: _run(e, cfg, 14, pexp) for e in (ENGINE_FULL, ENGINE_ORBIT, ENGINE_OCTANT)}
    ref = runs[ENGINE_FULL][1]
    for e in (ENGINE_ORBIT, ENGINE_OCTANT):
        for a, b in zip(runs[e][1], ref):
            assert abs(a["E"] - b["E"]) <= 1e-13 * abs(b["E"])
            assert np.max(np.abs(a["n"] - b["n"])) <= 1e-12 * np.max(np.abs(b["n"]))
        o, oref = runs[e][0], runs[ENGINE_FULL][0]
        for tp in range(o.window()[0], 17):
            assert np.allclose(o.F(16, tp), oref.F(16, tp), rtol=1e-13, atol=1e-15)
            assert np.allclose(o.rho(16, tp), oref.rho(16, tp), rtol=1e-13, atol=1e-15)


def test_full_lattice_keeps_cubic_symmetry():
    o, _ = _run(ENGINE_FULL, dict(Ns=6, M=5, dt=0.1, lam=4.0), 10)
    so = o.site_orbit()
    for tp in range(o.window()[0], 13):
        lat = o.lattice(0, 12, tp)
        for k in range(o.S):
            v = lat[so == k]
            assert np.ptp(v) <= 1e-13 * max(1.0, np.max(np.abs(lat)))


def test_lambda_zero_closed_form():
    """lambda = 0: Sigma = 0 and M^2 = m^2, so every F(t, t') and rho(t, t') obeys
    x_t = 2c x_{t-1} - x_{t-2}, c = 1 - w^2 dt^2 / 2 = cos(W dt), solved by
    x_t = x_1 U_{t-2}(c) - x_0 U_{t-3}(c) with U_n(cos a) = sin((n+1)a)/sin(a)."""
    dt, Ns, M, T = 0.1, 6, 40, 30
    o = Oracle(Ns, 3, M=M, N=4, dt=dt, lam=0.0, mass2=1.0, engine=ENGINE_OCTANT)
    _, k2, _ = o.orbits()
    n = 1.0 / (np.exp(np.sqrt(k2 + 1.0) / 2.0) - 1.0)
    o.init_occupation(n, 1.0)
    for t in range(3, T + 1):
        o.step(t)
    w2 = k2 + 1.0
    a = np.arccos(1 - w2 * dt * dt / 2)
    U = lambda m: np.sin((m + 1) * a) / np.sin(a)  # noqa: E731
    F11 = (n + 0.5) / np.sqrt(w2)
    F21 = F11
    for t in range(3, T + 1):
        # column t' = 1: x_1 = F(2,1), x_0 = F(1,1)
        Fc = F21 * U(t - 2) - F11 * U(t - 3)
        assert np.allclose(o.F(t, 1), Fc, rtol=1e-11, atol=1e-13)
        # rho(t, 1): x_0 = rho(1,1) = 0, x_1 = rho(2,1) = dt
        assert np.allclose(o.rho(t, 1), dt * U(t - 2), rtol=1e-11, atol=1e-13)
    assert abs(o.hartree_mass2(T, T) - 1.0) == 0.0


def test_gauss_energy_is_the_reference_formula():
    """Nx = 1 (0+1 dimensional) Gauss state: E(t=2) equals the conserved energy the
    reference prints (TwoPIScalar_Initialization.jl:109) and stays close to it.
    Parameters of Simulationfiles/Anders_NNLOpaper.jl:10-22 (600 steps, full memory)."""
    xi, eta, sig, lam, N, m2, dt = 0.4, 5.0, 1.0, 1.0, 8, 1.0, 0.01
    E0 = 0.5 * eta ** 2 + sig ** 2 / (8 * xi ** 2) + 0.5 * m2 * xi ** 2 + (1 / 24) * lam * (N + 2) / N * xi ** 4
    o = Oracle(1, 3, M=602, N=N, dt=dt, lam=lam, mass2=m2, engine=ENGINE_FULL)
    o.init_gauss(xi, eta, sig)
    assert abs(o.measure(2)["E"] - E0) <= 1e-12 * E0
    drift = 0.0
    for t in range(3, 603):
        o.step(t)
        drift = max(drift, abs(o.measure(t)["E"] - E0) / E0)
    assert drift < 2e-2


@pytest.mark.parametrize("name", ["small_ns8_m10", "c1_ns16_m202"])
def test_oracle_reproduces_golden(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    Ns, M, N, lam, dt, T, steps = g["cfg"]
    engine = ENGINE_FULL if name.startswith("small") else ENGINE_OCTANT
    o = Oracle(int(Ns), 3, M=int(M), N=int(N), dt=float(dt), lam=float(lam), engine=engine, nthreads=4)
    o.init_occupation(g["n0"], 1.0)
    scal = [list(o.measure(2)[k] for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2"))]
    for t in range(3, 3 + int(steps)):
        o.step(t)
        m = o.measure(t)
        scal.append([m[k] for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")])
    scal = np.array(scal)
    assert np.allclose(scal, g["scalars"], rtol=1e-12, atol=1e-14)


def test_gap_mass_newton():
    from kb2pi.twopiscalar import Discretization, Phi4, getGapMass

    o = Oracle(16, 3, M=4, N=4, lam=4.0, mass2=1.0)
    _, k2, deg = o.orbits()
    n = 5.0 * np.exp(-((np.sqrt(k2) - 1.0) ** 2) / (2 * 0.2 ** 2))
    m_or = o.gap_mass(n, 0.5)
    disc = Discretization(1.0, 16, 3, 0, 0.05, 16 ** 3, 1 / 16 ** 3, 4, 0)
    m_py = getGapMass(Phi4(4.0, 4, 1.0), "LambdaNLO", disc, n, k2, deg)
    assert abs(m_or - m_py) <= 1e-13
    # it solves the gap equation (TwoPIScalar_Initialization.jl:253-259)
    pref = 4.0 * 6 / 24
    g = np.sum((n + 0.5) * deg / np.sqrt(k2 + m_or ** 2)) / 16 ** 3 * pref + 1.0 - m_or ** 2
    assert abs(g) < 1e-12


def _loss_plain(cfg, n0, tf, wn, wE):
    o = make_oracle(cfg)
    o.init_occupation(n0, 1.0)
    for t in range(3, tf + 1):
        o.step(t)
    m = o.measure(tf)
    o.close()
    return float(np.dot(wn, m["n"]) + wE * m["E"])


@pytest.mark.parametrize("pexp", [1, 2, 0])
def test_dual_oracle_values_and_derivatives(pexp):
    """The dual-number engine reproduces the plain oracle's loss and its central
    finite differences (forward-mode derivatives pinned by FD on the oracle)."""
    from oracle.pyoracle import dual_loss

    cfg = dict(Ns=6, M=8, N=4, lam=2.0, dt=0.1, mass2=1.0, pexp=pexp)
    o = make_oracle(cfg)
    _, k2, deg = o.orbits()
    o.close()
    rng = np.random.default_rng(7 + pexp)
    n0 = thermal_n(k2, 1.5)
    wn = rng.random(len(k2)) * deg / deg.sum()
    dn = rng.random(len(k2))
    tf, wE = 20, 0.7
    L, dlam, dm2, ddn = dual_loss(cfg["Ns"], cfg["M"], n0, 1.0, tf, wn, wE, dn, N=4, dt=0.1, lam=2.0, mass2=1.0,
                                  pexp=pexp)
    L0 = _loss_plain(cfg, n0, tf, wn, wE)
    assert abs(L - L0) <= 1e-12 * abs(L0)
    h = 1e-5
    fl = (_loss_plain(dict(cfg, lam=2.0 + h * 2), n0, tf, wn, wE) - _loss_plain(dict(cfg, lam=2.0 - h * 2), n0, tf,
                                                                               wn, wE)) / (4 * h)
    fm = (_loss_plain(dict(cfg, mass2=1.0 + h), n0, tf, wn, wE) - _loss_plain(dict(cfg, mass2=1.0 - h), n0, tf, wn,
                                                                             wE)) / (2 * h)
    fn = (_loss_plain(cfg, n0 + h * dn, tf, wn, wE) - _loss_plain(cfg, n0 - h * dn, tf, wn, wE)) / (2 * h)
    assert abs(dlam - fl) <= 1e-6 * max(abs(fl), 1e-8) + 1e-10
    assert abs(dm2 - fm) <= 1e-6 * abs(fm)
    assert abs(ddn - fn) <= 1e-6 * abs(fn)


@pytest.mark.parametrize("Ns,M,steps", [(4, 6, 14), (6, 7, 12)])
@pytest.mark.parametrize("pexp", [4, 3])
def test_ninverse_engines_agree(Ns, M, steps, pexp):
    """1/N expansion: the literal full-lattice restatement of calcIrs!/calcIFs!/
    calcSelfEnergyattp! (CPUfull, with the reference's rfft/brfft pattern) and the
    orbit form (diagonal in momentum, triangular Volterra solves) agree."""
    res = []
    for eng in (ENGINE_FULL, ENGINE_OCTANT):
        o = Oracle(Ns, 3, M=M, N=4, dt=0.1, lam=4.0, mass2=1.0, pexp=pexp, engine=eng)
        _, k2, _ = o.orbits()
        o.init_occupation(thermal_n(k2, 2.0), 1.0)
        for t in range(3, steps + 3):
            o.step(t)
        res.append((o.measure(steps + 2), o.sigma(0, steps + 1) if pexp == 4 else None))
        o.close()
    (a, sa), (b, sb) = res
    assert np.max(np.abs(a["n"] - b["n"])) <= 1e-12 * np.max(np.abs(b["n"]))
    assert abs(a["E"] - b["E"]) <= 1e-12 * abs(b["E"])
    if pexp == 4:
        assert abs(b["E_mem"]) > 0
        assert np.max(np.abs(sa - sb)) <= 1e-12 * np.max(np.abs(sb))


def test_ninverse_energy_drift_matches_lambda_nlo_scale():
    """A 1/N NLO run conserves energy to the same order as the lambda expansion."""
    drifts = []
    for pexp in (1, 4):
        o = Oracle(6, 3, M=60, N=4, dt=0.05, lam=2.0, mass2=1.0, pexp=pexp, engine=ENGINE_OCTANT)
        _, k2, _ = o.orbits()
        o.init_occupation(thermal_n(k2, 1.5), 1.0)
        E = []
        for t in range(3, 123):
            o.step(t)
            if t % 20 == 0:
                E.append(o.measure(t)["E"])
        o.close()
        drifts.append(abs(E[-1] - E[0]) / abs(E[0]))
    assert drifts[1] < 5e-3
