"""kb_adjoint (discrete adjoint of the KB step) against central finite
differences of the FP64 GPU forward run and of the CPU oracle.

The loss is L = sum_k w_n[k] n(k, t_f) + w_E E(t_f). Tolerance: 1e-4 relative
(max |adjoint - FD| / max |FD| over each gradient), with FD steps of 1e-5
relative; the window is shorter than the run, so rows leave the ring and the
reverse sweep crosses several recomputed checkpoint blocks.
"""
import numpy as np
import pytest

from kbtest_util import make_gpu, make_oracle, occupation, rel

pytestmark = pytest.mark.gpu

TOL = 1e-4
BASE = dict(Ns=6, M=12, N=4, lam=2.0, dt=0.1, mass2=1.0, mass=1.0, T=1.5, pexp=1)


def gpu_loss(cfg, n0, tf, wn, wE, init_mass=1.0):
    h = make_gpu(dict(cfg, flags=0))
    try:
        h.init(0, n0, init_mass)
        for t in range(3, tf + 1):
            h.step(t)
        m = h.measure(0, tf)
        return float(np.dot(wn, m["n"]) + wE * m["E"])
    finally:
        h.close()


def oracle_loss(cfg, n0, tf, wn, wE, init_mass=1.0):
    o = make_oracle(cfg)
    o.init_occupation(n0, init_mass)
    for t in range(3, tf + 1):
        o.step(t)
    m = o.measure(tf)
    return float(np.dot(wn, m["n"]) + wE * m["E"])


def central(f, x, rel_h=1e-5):
    h = rel_h * max(abs(x), 1.0)
    return (f(x + h) - f(x - h)) / (2 * h)


def setup(cfg, seed):
    g = make_gpu(dict(cfg, flags=0))
    _, k2, deg = g.orbits()
    g.close()
    rng = np.random.default_rng(seed)
    n0 = occupation(cfg, k2)
    wn = rng.random(len(k2)) * deg / deg.sum()
    return k2, deg, n0, wn


def adjoint(cfg, n0, tf, wn, wE, ckpt, init_mass=1.0):
    h = make_gpu(dict(cfg, flags=ckpt))
    try:
        return h.adjoint(n0, init_mass, tf, w_n=wn, w_E=wE, ckpt_every=ckpt)
    finally:
        h.close()


@pytest.mark.parametrize("pexp", [1, 2, 0])
def test_adjoint_matches_finite_differences(pexp):
    cfg = dict(BASE, pexp=pexp)
    tf, wE, ckpt = 30, 0.7, 5
    k2, deg, n0, wn = setup(cfg, 11 + pexp)
    g = adjoint(cfg, n0, tf, wn, wE, ckpt)
    L = gpu_loss(cfg, n0, tf, wn, wE)
    assert abs(g["loss"] - L) <= 1e-12 * abs(L)
    fd_lam = central(lambda v: gpu_loss(dict(cfg, lam=v), n0, tf, wn, wE), cfg["lam"])
    fd_m2 = central(lambda v: gpu_loss(dict(cfg, mass2=v), n0, tf, wn, wE), cfg["mass2"])
    fd_mi = central(lambda v: gpu_loss(cfg, n0, tf, wn, wE, init_mass=v), 1.0)
    fd_n = np.zeros(len(n0))
    for q in range(len(n0)):
        def f(v, q=q):
            x = n0.copy()
            x[q] = v
            return gpu_loss(cfg, x, tf, wn, wE)
        fd_n[q] = central(f, n0[q])
    if pexp == 0:
        assert abs(g["lambda"] - fd_lam) <= TOL * max(abs(fd_lam), 1e-12)
    else:
        assert rel(g["lambda"], fd_lam) <= TOL
    assert rel(g["mass2"], fd_m2) <= TOL
    assert rel(g["init_mass"], fd_mi) <= TOL
    assert rel(g["n_init"], fd_n) <= TOL


def test_adjoint_checkpoint_interval_does_not_change_gradients():
    cfg = dict(BASE)
    tf, wE = 27, 1.0
    _, _, n0, wn = setup(cfg, 5)
    a = adjoint(cfg, n0, tf, wn, wE, 1)
    b = adjoint(cfg, n0, tf, wn, wE, 7)
    c = adjoint(cfg, n0, tf, wn, wE, 40)  # one block: no recomputation
    for x in (b, c):
        assert rel(x["n_init"], a["n_init"]) <= 1e-12
        assert abs(x["lambda"] - a["lambda"]) <= 1e-12 * abs(a["lambda"])
        assert abs(x["mass2"] - a["mass2"]) <= 1e-12 * abs(a["mass2"])


def test_adjoint_matches_oracle_finite_differences():
    """The CPU FP64 oracle's own FD of the same loss (it shares no code with the
    adjoint or the GPU forward)."""
    cfg = dict(BASE, Ns=8, M=10, lam=3.0)
    tf, wE, ckpt = 24, 0.5, 4
    _, _, n0, wn = setup(cfg, 3)
    g = adjoint(cfg, n0, tf, wn, wE, ckpt)
    fd_lam = central(lambda v: oracle_loss(dict(cfg, lam=v), n0, tf, wn, wE), cfg["lam"])
    fd_m2 = central(lambda v: oracle_loss(dict(cfg, mass2=v), n0, tf, wn, wE), cfg["mass2"])
    assert rel(g["lambda"], fd_lam) <= TOL
    assert rel(g["mass2"], fd_m2) <= TOL
    # a directional derivative along a random occupation perturbation
    d = np.random.default_rng(9).random(len(n0))
    fd_dir = central(lambda s: oracle_loss(cfg, n0 + s * d, tf, wn, wE), 0.0)
    assert rel(np.dot(g["n_init"], d), fd_dir) <= TOL


def test_adjoint_errors():
    from kb2pi import capi

    cfg = dict(BASE)
    _, _, n0, wn = setup(cfg, 1)
    h = make_gpu(dict(cfg, flags=2))
    with pytest.raises(capi.KbError, match="extra ring slots"):
        h.adjoint(n0, 1.0, 20, w_n=wn, w_E=1.0, ckpt_every=5)
    with pytest.raises(capi.KbError, match="t_final"):
        h.adjoint(n0, 1.0, 2, w_n=wn, w_E=1.0, ckpt_every=2)
    h.close()
    h = make_gpu(dict(cfg, flags=5), precision=1)
    with pytest.raises(capi.KbError, match="FP64"):
        h.adjoint(n0, 1.0, 20, w_n=wn, w_E=1.0, ckpt_every=5)
    h.close()


def test_extra_ring_slots_leave_the_forward_unchanged():
    cfg = dict(BASE, M=10)
    _, _, n0, _ = setup(cfg, 2)
    out = []
    for flags in (0, 9):
        h = make_gpu(dict(cfg, flags=flags))
        h.init(0, n0, 1.0)
        for t in range(3, 40):
            h.step(t)
        m = h.measure(0, 39)
        out.append((m["n"], m["E"], h.get(0, 0, 39, 31)))
        h.close()
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])


def test_torch_function_backward():
    torch = pytest.importorskip("torch")
    from kb2pi import adjoint as adj

    cfg = dict(BASE)
    g = make_gpu(dict(cfg, flags=0))
    _, k2, deg = g.orbits()
    g.close()
    B = adj.bump_basis(k2, 8)
    wn = adj.shell_weights(k2, deg, 8)
    amps = torch.tensor(np.random.default_rng(4).uniform(0, 5, 8), dtype=torch.float64, requires_grad=True)
    lam = torch.tensor(2.0, dtype=torch.float64, requires_grad=True)
    m2 = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    KBLoss = adj.make_function()
    L = KBLoss.apply(lam, m2, amps, cfg, B, 20, wn, 1.0, 5)
    L.backward()
    n0 = amps.detach().numpy() @ B
    assert abs(L.item() - gpu_loss(cfg, n0, 20, wn, 1.0)) <= 1e-12 * abs(L.item())
    fd = central(lambda v: gpu_loss(dict(cfg, lam=v), n0, 20, wn, 1.0), 2.0)
    assert rel(lam.grad.item(), fd) <= TOL
    e = np.zeros(8)
    e[3] = 1.0
    fd_a = central(lambda s: gpu_loss(cfg, (amps.detach().numpy() + s * e) @ B, 20, wn, 1.0), 0.0)
    assert rel(amps.grad[3].item(), fd_a) <= TOL


@pytest.mark.parametrize("pexp", [1, 2, 0])
def test_adjoint_matches_dual_number_oracle(pexp):
    """Exact derivatives on both sides: the GPU adjoint against forward-mode dual
    numbers through the CPU oracle (the stand-in for ForwardDiff through the
    reference), to 1e-8 relative -- far below what finite differences resolve."""
    from oracle.pyoracle import dual_loss

    cfg = dict(BASE, Ns=8, M=9, lam=2.5, pexp=pexp)
    tf, wE, ckpt = 26, 0.6, 4
    _, _, n0, wn = setup(cfg, 21 + pexp)
    dn = np.random.default_rng(31).random(len(n0)) - 0.3
    g = adjoint(cfg, n0, tf, wn, wE, ckpt)
    L, dlam, dm2, ddn = dual_loss(cfg["Ns"], cfg["M"], n0, 1.0, tf, wn, wE, dn, N=cfg["N"], dt=cfg["dt"],
                                  lam=cfg["lam"], mass2=cfg["mass2"], pexp=pexp)
    assert abs(g["loss"] - L) <= 1e-11 * abs(L)
    assert abs(g["lambda"] - dlam) <= 1e-8 * abs(dlam) + 1e-12
    assert abs(g["mass2"] - dm2) <= 1e-8 * abs(dm2)
    assert abs(np.dot(g["n_init"], dn) - ddn) <= 1e-8 * abs(ddn)
