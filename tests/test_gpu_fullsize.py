"""The largest and smallest sizes the library accepts, and the headline workload
itself (Ns = 64, memory window M = 1000, the window wrapped), checked through
properties that hold at any size:

- lambda = 0: Sigma = 0 and M^2 = m^2, so every F(t, t') and rho(t, t') is the
  bilinear closed form of the linear recurrence x_t = 2c x_{t-1} - x_{t-2},
  c = 1 - w^2 dt^2 / 2, in both time arguments, from F(1,1), F(2,1), F(2,2) and
  rho(2,1) = dt (the known answer of TwoPIScalar_Evolution.jl:890-915 with
  Sigma = 0); U_n(cos a) = sin((n+1)a) / sin(a);
- structural invariants rho(t,t) = 0 and rho(t,t-1) = dt (Evolution.jl:891-896);
- FP64 and mixed precision agree within 1e-5 on n and E at the headline size;
- the sunset on the largest lattice against the FP64 oracle (random rows, the
  fast-vs-simple pattern of TwoPIScalar_Tests_LambdaNLO_checkfastimplementation.jl);
- the smallest lattices and the smallest window against the FP64 oracle.
"""
import numpy as np
import pytest

from kbtest_util import make_gpu, make_oracle, occupation, random_symmetric_row, rel

pytestmark = pytest.mark.gpu


def _closed_form(k2, mass2, dt, F11, F21, F22):
    """F(t, t') and rho(t, t') at lambda = 0 as functions of (t, t')."""
    w2 = np.asarray(k2) + mass2
    a = np.arccos(1.0 - w2 * dt * dt / 2.0)

    def U(n):
        return np.sin((n + 1) * a) / np.sin(a)

    def u(t):  # x_t = x_2 u2(t) + x_1 u1(t)
        return U(t - 2), -U(t - 3)

    def F(t, tp):
        a2, a1 = u(t)
        b2, b1 = u(tp)
        return a2 * b2 * F22 + a2 * b1 * F21 + a1 * b2 * F21 + a1 * b1 * F11

    def rho(t, tp):  # rho(1,1) = rho(2,2) = 0, rho(2,1) = dt = -rho(1,2)
        a2, a1 = u(t)
        b2, b1 = u(tp)
        return dt * (a2 * b1 - a1 * b2)

    return F, rho


@pytest.mark.parametrize("Ns,M,steps,precision", [
    (64, 1000, 1008, 0),   # the headline lattice and window, wrapped: t = 1010, tmin = 11
    (64, 1000, 1008, 1),
    (8, 1024, 1100, 0),    # the largest window
    (8, 1024, 1100, 1),
])
def test_lambda_zero_closed_form_at_full_size(Ns, M, steps, precision):
    dt, mass2 = 0.05, 1.0
    cfg = dict(Ns=Ns, M=M, dt=dt, lam=0.0, T=2.0, mass2=mass2)
    h = make_gpu(cfg, precision)
    _, k2, _ = h.orbits(0)
    h.init(0, occupation(cfg, k2), 1.0)
    F11, F21, F22 = h.get(0, 0, 1, 1), h.get(0, 0, 2, 1), h.get(0, 0, 2, 2)
    assert np.all(h.get(0, 1, 2, 1) == dt)
    F, rho = _closed_form(k2, mass2, dt, F11, F21, F22)
    h.steps(3, steps, 0)
    t = 2 + steps
    tmin, tmax = h.window(0)
    assert tmax == t and tmin == max(1, t - M + 1)
    # the state rows t, t-1 are FP64 in both precisions; older rows of the mixed
    # form come from the FP32 history
    for a in (t, t - 1, (tmin + t) // 2):
        tol = 1e-9 if (precision == 0 or a >= t - 1) else 3e-7
        for tp in sorted({tmin, tmin + 1, (tmin + a) // 2, a - 1, a}):
            assert rel(h.get(0, 0, a, tp), F(a, tp)) <= tol, (a, tp)
            if tp < a:
                assert rel(h.get(0, 1, a, tp), rho(a, tp)) <= tol, (a, tp)
    assert np.all(h.get(0, 1, t, t) == 0.0)
    assert np.all(h.get(0, 1, t, t - 1) == dt)
    m = h.measure(0, t)
    assert m["M2"] == mass2
    h.close()


def test_headline_size_mixed_matches_fp64():
    """Ns = 64, M = 1000, tsunami, lambda = 2 (the headline workload) through the
    first wrap of the window: mixed precision within 1e-5 of plain FP64 on n
    per orbit and E, and on the newest row of F."""
    cfg = dict(Ns=64, M=1000, dt=0.05, lam=2.0, init="tsunami")
    steps = 1008
    out = []
    for precision in (0, 1):
        h = make_gpu(cfg, precision)
        _, k2, _ = h.orbits(0)
        h.init(0, occupation(cfg, k2), 1.0)
        h.steps(3, steps, 0)
        t = 2 + steps
        out.append((h.measure(0, t), h.get(0, 0, t, t - 500)))
        h.close()
    (m64, row64), (mmx, rowmx) = out
    assert rel(mmx["n"], m64["n"]) <= 1e-5
    assert abs(mmx["E"] - m64["E"]) <= 1e-5 * abs(m64["E"])
    assert rel(rowmx, row64) <= 1e-5


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-5)])
def test_largest_lattice_sunset_matches_oracle(precision, tol):
    """Sigma(t-1, t') at Ns = 64 for random cubic-symmetric rows: the GPU orbit
    cosine transforms against the oracle's FP64 transforms."""
    cfg = dict(Ns=64, M=14, dt=0.01, lam=10.0, N=8, T=2.0)
    g = make_gpu(cfg, precision)
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
    t = 11
    tmone = t - 1
    rng = np.random.default_rng(64)
    for tp in range(1, t):
        Fv, rv = random_symmetric_row(g.S[0], rng), random_symmetric_row(g.S[0], rng)
        if tp == tmone:
            rv[:] = 0.0
        g.set(0, 0, tmone, tp, Fv)
        g.set(0, 1, tmone, tp, rv)
        o.set(0, tmone, tp, Fv)
        o.set(1, tmone, tp, rv)
    g.self_energies(tmone)
    o.self_energies(tmone)
    for tp in range(1, t):
        assert rel(g.sigma(0, 1, tp), o.sigma(1, tp)) <= tol, tp
        assert rel(g.sigma(0, 0, tp), o.sigma(0, tp)) <= tol, tp
    g.close()


@pytest.mark.parametrize("Ns,M", [(2, 3), (4, 3), (2, 7)])
@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-5)])
def test_smallest_sizes_follow_oracle(Ns, M, precision, tol):
    """The smallest lattices (one and two octant points per axis) and the
    smallest window (M = 3: the ring wraps every step)."""
    cfg = dict(Ns=Ns, M=M, dt=0.1, lam=2.0, T=2.0)
    g = make_gpu(cfg, precision)
    o = make_oracle(cfg)
    _, k2, _ = g.orbits(0)
    n = occupation(cfg, k2)
    g.init(0, n, 1.0)
    o.init_occupation(n, 1.0)
    for t in range(3, 40):
        g.step(t)
        o.step(t)
        mg, mo = g.measure(0, t), o.measure(t)
        assert abs(mg["E"] - mo["E"]) <= tol * abs(mo["E"]), t
        assert rel(mg["n"], mo["n"]) <= tol, t
    tmin, tmax = g.window(0)
    assert (tmin, tmax) == o.window()
    for tp in range(tmin, tmax + 1):
        assert rel(g.get(0, 0, tmax, tp), o.F(tmax, tp)) <= tol
    g.close()
