"""Launch tuning (kb_get_tuning / kb_set_tuning / kb_autotune): every
configuration computes the same step. Sunset grids are bitwise identical (one
CTA per row whatever the grid); the two FP32 memory-integral variants differ
only in the order of FP32 tile partial sums; the autotuner re-runs the last
step and leaves the state as a plain run would."""
import numpy as np
import pytest

from kbtest_util import make_gpu, occupation, rel

pytestmark = pytest.mark.gpu

CFG = dict(Ns=12, M=40, N=4, lam=3.0, dt=0.1, mass2=1.0, pexp=1, T=1.5)


def evolve(cfg, precision, steps, tuning=None, autotune_at=None):
    h = make_gpu(cfg, precision)
    _, k2, _ = h.orbits()
    h.init(0, occupation(cfg, k2), 1.0)
    if tuning:
        h.set_tuning(**tuning)
    for t in range(3, steps + 3):
        h.step(t)
        if t == autotune_at:
            h.autotune(trials=2)
    m = h.measure(0, steps + 2)
    row = h.get(0, 0, steps + 2, steps - 20)
    h.close()
    return m, row


@pytest.mark.parametrize("precision", [0, 1])
def test_sunset_grids_are_bitwise_identical(precision):
    h = make_gpu(CFG, precision)
    sms = h.tuning()["sunset_grid"]
    h.close()
    a = evolve(CFG, precision, 60)
    b = evolve(CFG, precision, 60, tuning={"sunset_grid": 2 * sms if sms < 38 else sms})
    c = evolve(CFG, precision, 60, tuning={"sunset_grid": 7})
    for x in (b, c):
        assert np.array_equal(x[0]["n"], a[0]["n"]) and x[0]["E"] == a[0]["E"]
        assert np.array_equal(x[1], a[1])


def test_memint_variants_agree():
    a = evolve(CFG, 1, 60, tuning={"memint_variant": 0})
    b = evolve(CFG, 1, 60, tuning={"memint_variant": 1})
    assert rel(a[0]["n"], b[0]["n"]) <= 1e-6
    assert abs(a[0]["E"] - b[0]["E"]) <= 1e-6 * abs(b[0]["E"])


def test_autotune_keeps_the_state_fp64():
    a = evolve(CFG, 0, 60)
    b = evolve(CFG, 0, 60, autotune_at=30)
    assert np.array_equal(a[0]["n"], b[0]["n"]) and a[0]["E"] == b[0]["E"]
    assert np.array_equal(a[1], b[1])


def test_autotune_mixed_and_errors():
    from kb2pi import capi

    b = evolve(CFG, 1, 60, autotune_at=30)
    a = evolve(CFG, 1, 60)
    assert rel(a[0]["n"], b[0]["n"]) <= 1e-6
    h = make_gpu(CFG, 0)
    with pytest.raises(capi.KbError, match="t >= 3"):
        h.autotune()
    with pytest.raises(capi.KbError, match="memint_variant"):
        h.set_tuning(memint_variant=1)
    with pytest.raises(capi.KbError, match="sunset_grid"):
        h.set_tuning(sunset_grid=10 ** 6)
    h.close()
