"""Launch tuning (kb_get_tuning / kb_set_tuning / kb_autotune): every
configuration computes the same step. Sunset grids are bitwise identical (one
CTA per row whatever the grid); the two FP32 memory-integral variants differ
only in the order of FP32 tile partial sums; the autotuner re-runs the last
step and leaves the state as a plain run would."""
import time

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
    """One CTA per sunset item (FP64: a t' row; FP32 at Ns = 12: eight rows) whatever
    the grid, so every grid gives the same bits."""
    h = make_gpu(CFG, precision)
    items = h.tuning()["sunset_grid"]  # one CTA per item by default at this size
    h.close()
    a = evolve(CFG, precision, 60)
    b = evolve(CFG, precision, 60, tuning={"sunset_grid": max(1, items // 2)})
    c = evolve(CFG, precision, 60, tuning={"sunset_grid": 1})
    runs = [b, c]
    if precision == 1:  # the 512-thread FP32 sunset computes every element the same way
        runs.append(evolve(CFG, precision, 60, tuning={"sunset_variant": 1, "sunset_grid": max(1, items - 1)}))
    for x in runs:
        assert np.array_equal(x[0]["n"], a[0]["n"]) and x[0]["E"] == a[0]["E"]
        assert np.array_equal(x[1], a[1])


def test_sunset_items_of_several_rows_are_bitwise_identical():
    """FP32 runs of small lattices put several t' rows in one sunset item (Ns = 8,
    10, 16: 8 rows, 24: 4), windows of 23..41 rows leave partial last items; with
    every sunset variant and grid each run of the batch gives the bits of the same
    run alone."""
    from kb2pi import capi

    cfgs = [dict(Ns=24, M=30, lam=2.0, T=1.0), dict(Ns=8, M=41, lam=4.0, T=2.0), dict(Ns=16, M=37, lam=1.0, T=0.7),
            dict(Ns=10, M=23, lam=3.0, T=1.5)]

    def params(c):
        return capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=1, device=0, flags=0, dt=0.1,
                             lam=c["lam"], mass2=1.0, mass=1.0)

    out = []
    for variant, grid in ((0, 0), (1, 0), (1, 5)):
        h = capi.Handle([params(c) for c in cfgs])
        for r, c in enumerate(cfgs):
            _, k2, _ = h.orbits(r)
            h.init(r, occupation(dict(c), k2), 1.0)
        h.set_tuning(sunset_variant=variant, sunset_grid=grid)
        h.steps(3, 50, 0)
        out.append([h.measure(r, 52) for r in range(len(cfgs))])
        h.close()
    for r, c in enumerate(cfgs):  # each run alone
        g = make_gpu(dict(c, dt=0.1), 1)
        _, k2, _ = g.orbits()
        g.init(0, occupation(dict(c), k2), 1.0)
        g.steps(3, 50, 0)
        m = g.measure(0, 52)
        g.close()
        for o in out:
            assert o[r]["E"] == m["E"] and np.array_equal(o[r]["n"], m["n"]), r


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
    with pytest.raises(capi.KbError, match="sunset_variant"):
        h.set_tuning(sunset_variant=1)
    h.close()


def test_batch_orders_are_bitwise_identical():
    """Reordering the runs' CTA ranges changes which CTA computes what, not how."""
    from kb2pi import capi

    cfgs = [dict(Ns=8, M=20, lam=2.0, T=1.0), dict(Ns=16, M=45, lam=4.0, T=2.0), dict(Ns=12, M=33, lam=1.0, T=0.7)]
    out = []
    for order in (0, 1):
        ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=1, device=0, flags=0, dt=0.1,
                            lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
        h = capi.Handle(ps)
        for r, c in enumerate(cfgs):
            _, k2, _ = h.orbits(r)
            h.init(r, occupation(dict(c), k2), 1.0)
        h.set_tuning(batch_order=order)
        assert h.tuning()["batch_order"] == order
        h.steps(3, 60, 0)
        out.append([h.measure(r, 62)["n"] for r in range(3)])
        if order == 1:
            d = h.autotune(trials=1)
            assert d["batch_order"] in (0, 1)
        h.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("pexp", [1, 0, 4])
def test_memint_split_matches_oracle_fp64(pexp):
    """Split memory integrals (two half-triangle CTAs per chunk + finishing
    kernel) against the FP64 oracle: 1e-10, the plain path's bound; the window
    wraps so both halves and the ring edges are exercised."""
    from kbtest_util import make_oracle

    cfg = dict(Ns=8, M=23, N=4, lam=3.0, dt=0.1, mass2=1.0, pexp=pexp, T=1.5)
    g = make_gpu(cfg, 0)
    o = make_oracle(cfg)
    _, k2, _ = g.orbits()
    n0 = occupation(cfg, k2)
    g.init(0, n0, 1.0)
    o.init_occupation(n0, 1.0)
    g.set_tuning(memint_split=1)
    assert g.tuning()["memint_split"] == 1
    for t in range(3, 63):
        g.step(t)
        o.step(t)
        if t % 10 == 2:
            mg, mo = g.measure(0, t), o.measure(t)
            assert rel(mg["n"], mo["n"]) <= 1e-10
            assert abs(mg["E"] - mo["E"]) <= 1e-10 * abs(mo["E"])
            tp = max(g.window(0)[0], t - 15)
            assert rel(g.get(0, 0, t, tp), o.F(t, tp)) <= 1e-10
    g.close()
    o.close()


def test_memint_split_mixed_and_batched():
    from kb2pi import capi

    a = evolve(CFG, 1, 60, tuning={"memint_split": 0})
    b = evolve(CFG, 1, 60, tuning={"memint_split": 1})
    assert rel(a[0]["n"], b[0]["n"]) <= 1e-6
    assert abs(a[0]["E"] - b[0]["E"]) <= 1e-6 * abs(a[0]["E"])
    # a batched FP64 handle in split mode equals its single runs to rounding
    cfgs = [dict(Ns=8, M=20, lam=2.0, T=1.0), dict(Ns=12, M=37, lam=4.0, T=2.0)]
    ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=0, device=0, flags=0, dt=0.1,
                        lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
    hb = capi.Handle(ps)
    hs = [capi.Handle([p]) for p in ps]
    for r, c in enumerate(cfgs):
        _, k2, _ = hb.orbits(r)
        hb.init(r, occupation(dict(c), k2), 1.0)
        hs[r].init(0, occupation(dict(c), k2), 1.0)
    hb.set_tuning(memint_split=1, batch_order=1)
    hb.steps(3, 50, 0)
    for r, h in enumerate(hs):
        h.steps(3, 50, 0)
        x, y = hb.measure(r, 52), h.measure(0, 52)
        assert rel(x["n"], y["n"]) <= 1e-10 and abs(x["E"] - y["E"]) <= 1e-10 * abs(y["E"])
    for h in [hb] + hs:
        h.close()
    h = make_gpu(CFG, 1)
    with pytest.raises(capi.KbError, match="memint_split"):
        h.set_tuning(memint_variant=0, memint_split=1)
    h.close()


@pytest.mark.parametrize("precision,tol,Ns,variant", [(0, 1e-10, 40, 1), (1, 1e-6, 40, 1), (0, 1e-10, 36, 1),
                                                      (1, 1e-6, 36, 2), (1, 1e-6, 38, 2), (0, 1e-10, 38, 1)])
def test_memint_tail_split_matches_whole(precision, tol, Ns, variant):
    """memint_split 2 at Ns = 36, 38, 40 (167, 193, 222 chunks): the chunks of the
    whole waves of one CTA per SM stream whole, the rest in parts (6, 3 and 2 parts
    on 152 SMs: as many as fill the last wave best) that the finishing kernel
    completes; F, rho, n and E agree with the whole-chunk kernel (FP64 to 1e-10,
    mixed to 1e-6) with the window wrapped."""
    cfg = dict(Ns=Ns, M=20, N=4, lam=3.0, dt=0.1, pexp=1, T=1.5)
    hs = []
    for split in (0, 2):
        h = make_gpu(cfg, precision)
        _, k2, _ = h.orbits()
        h.init(0, occupation(cfg, k2), 1.0)
        if precision == 1:
            h.set_tuning(memint_variant=variant, memint_split=split)
        else:
            h.set_tuning(memint_split=split)
        assert h.tuning()["memint_split"] == split
        h.steps(3, 30, 0)
        hs.append(h)
    a, b = hs
    ma, mb = a.measure(0, 32), b.measure(0, 32)
    assert rel(mb["n"], ma["n"]) <= tol
    assert abs(mb["E"] - ma["E"]) <= tol * abs(ma["E"])
    for tp in (13, 20, 31, 32):
        assert rel(b.get(0, 0, 32, tp), a.get(0, 0, 32, tp)) <= tol
        assert rel(b.get(0, 1, 32, tp), a.get(0, 1, 32, tp)) <= tol
    for h in hs:
        h.close()


@pytest.mark.parametrize("cfg,split", [
    (dict(Ns=40, M=20, N=4, lam=3.0, dt=0.1, pexp=1, T=1.5), 0),   # 222 chunks, window wrapped
    (dict(Ns=40, M=20, N=4, lam=3.0, dt=0.1, pexp=1, T=1.5), 2),   # whole waves with leapfrog warps, tail split
    (dict(Ns=12, M=40, N=4, lam=3.0, dt=0.1, pexp=2, T=1.5), 0),   # classical sunset, one partial wave
    (dict(Ns=10, M=30, N=4, lam=3.0, dt=0.1, pexp=0, T=1.5), 0),   # LO: no memory integral, leapfrog only
])
def test_leapfrog_warps_are_bitwise_identical(cfg, split):
    """memint_variant 2 (whole chunks hand each column block's sums to four
    leapfrog warps) runs the same leapfrog arithmetic in the same order as the
    column group of variant 1: F, rho, n and E agree bitwise."""
    hs = []
    for variant in (1, 2):
        h = make_gpu(cfg, 1)
        _, k2, _ = h.orbits()
        h.init(0, occupation(cfg, k2), 1.0)
        h.set_tuning(memint_variant=variant, memint_split=split)
        assert h.tuning()["memint_variant"] == variant
        h.steps(3, 30, 0)
        for t in range(33, 36):  # single steps after the graph-captured ones
            h.step(t)
        hs.append(h)
    a, b = hs
    ma, mb = a.measure(0, 35), b.measure(0, 35)
    assert ma["E"] == mb["E"] and np.array_equal(ma["n"], mb["n"])
    tmin, _ = a.window(0)
    for tp in sorted({tmin, (tmin + 35) // 2, 34, 35}):
        assert np.array_equal(a.get(0, 0, 35, tp), b.get(0, 0, 35, tp))
        assert np.array_equal(a.get(0, 1, 35, tp), b.get(0, 1, 35, tp))
    for h in hs:
        h.close()


def test_leapfrog_warps_batched_runs():
    """Batched uneven runs with the leapfrog warps: bitwise equal to variant 1."""
    from kb2pi import capi

    cfgs = [dict(Ns=8, M=20, lam=2.0, T=1.0), dict(Ns=16, M=45, lam=4.0, T=2.0), dict(Ns=12, M=33, lam=1.0, T=0.7)]
    out = []
    for variant in (1, 2):
        ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=1, device=0, flags=0, dt=0.1,
                            lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
        h = capi.Handle(ps)
        for r, c in enumerate(cfgs):
            _, k2, _ = h.orbits(r)
            h.init(r, occupation(dict(c), k2), 1.0)
        h.set_tuning(memint_variant=variant)
        h.steps(3, 60, 0)
        out.append([h.measure(r, 62) for r in range(3)])
        h.close()
    for a, b in zip(out[0], out[1]):
        assert a["E"] == b["E"] and np.array_equal(a["n"], b["n"])


@pytest.mark.parametrize("precision,M", [(0, 40), (1, 40), (1, 100)])
def test_memint_bulk_copies_match_tensor_maps(precision, M):
    """History tiles by plain bulk copies (memint_bulk 1, the path without a
    tensor-map encoder) give the same F, rho, n and E as the tensor-map boxes,
    bitwise: both deliver the same bytes in the same stage layout. M = 100 puts
    whole FP32 diagonal tiles inside the window, whose upper-right quadrants
    neither path loads."""
    cfg = dict(Ns=12, M=M, N=4, lam=3.0, dt=0.1, pexp=1, T=1.5)
    hs = []
    for bulk in (0, 1):
        h = make_gpu(cfg, precision)
        _, k2, _ = h.orbits()
        h.init(0, occupation(cfg, k2), 1.0)
        h.set_tuning(memint_bulk=bulk)
        assert h.tuning()["memint_bulk"] == bulk
        h.steps(3, 70, 0)
        hs.append(h)
    a, b = hs
    ma, mb = a.measure(0, 72), b.measure(0, 72)
    assert ma["E"] == mb["E"] and np.array_equal(ma["n"], mb["n"])
    for tp in (33, 50, 72):
        assert np.array_equal(a.get(0, 0, 72, tp), b.get(0, 0, 72, tp))
        assert np.array_equal(a.get(0, 1, 72, tp), b.get(0, 1, 72, tp))
    for h in hs:
        h.close()


@pytest.mark.parametrize("precision,variant,split", [(0, 0, 0), (0, 0, 1), (1, 1, 0), (1, 1, 1), (1, 2, 0), (1, 2, 2)])
def test_persistent_memint_is_bitwise_the_grid_of_one_cta_per_item(precision, variant, split):
    """memint_persistent 1 (one CTA per SM taking chunk items from a queue, its stage
    barriers' phases running on across items, the tadpole sum kept per run) gives the
    same F, rho, n and E as one CTA per item, bitwise; 222 chunks at Ns = 40, more
    than one per SM, so CTAs take several items (and split halves with split 1, 2)."""
    cfg = dict(Ns=40, M=20, N=4, lam=3.0, dt=0.1, pexp=1, T=1.5)
    hs = []
    for pers in (0, 1):
        h = make_gpu(cfg, precision)
        _, k2, _ = h.orbits()
        h.init(0, occupation(cfg, k2), 1.0)
        h.set_tuning(memint_variant=variant, memint_split=split, memint_persistent=pers)
        assert h.tuning()["memint_persistent"] == pers
        h.steps(3, 30, 0)
        for t in range(33, 36):  # single steps after the graph-captured ones
            h.step(t)
        hs.append(h)
    a, b = hs
    ma, mb = a.measure(0, 35), b.measure(0, 35)
    assert ma["E"] == mb["E"] and np.array_equal(ma["n"], mb["n"])
    tmin, _ = a.window(0)
    for tp in sorted({tmin, (tmin + 35) // 2, 34, 35}):
        assert np.array_equal(a.get(0, 0, 35, tp), b.get(0, 0, 35, tp))
        assert np.array_equal(a.get(0, 1, 35, tp), b.get(0, 1, 35, tp))
    for h in hs:
        h.close()


def test_persistent_memint_batched_runs_and_errors():
    """Uneven batched runs (several runs per CTA, tadpole sums switching between
    runs) bitwise equal with and without the persistent grid; the register-blocked
    kernel has no persistent form; the autotuner reports its choice."""
    from kb2pi import capi

    cfgs = [dict(Ns=24, M=30, lam=2.0, T=1.0), dict(Ns=8, M=41, lam=4.0, T=2.0), dict(Ns=16, M=37, lam=1.0, T=0.7),
            dict(Ns=6, M=9, lam=3.0, T=1.5), dict(Ns=24, M=20, lam=1.0, T=1.0)]
    out = []
    for pers in (0, 1):
        ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=1, device=0, flags=0, dt=0.1,
                            lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
        h = capi.Handle(ps)
        for r, c in enumerate(cfgs):
            _, k2, _ = h.orbits(r)
            h.init(r, occupation(dict(c), k2), 1.0)
        h.set_tuning(memint_variant=2, memint_split=1, batch_order=1, memint_persistent=pers)
        h.steps(3, 50, 0)
        out.append([(h.measure(r, 52), h.get(r, 0, 52, 48), h.get(r, 1, 52, 48)) for r in range(len(cfgs))])
        if pers:
            with pytest.raises(capi.KbError, match="KB_ERR_PARAM"):
                h.set_tuning(memint_variant=0, memint_split=0, memint_persistent=1)
            chosen = h.autotune(trials=1)
            assert chosen["memint_persistent"] in (0, 1)
        h.close()
    for (ma, Fa, ra), (mb, Fb, rb) in zip(out[0], out[1]):
        assert ma["E"] == mb["E"] and np.array_equal(ma["n"], mb["n"])
        assert np.array_equal(Fa, Fb) and np.array_equal(ra, rb)


@pytest.mark.parametrize("split", [0, 2])
def test_persistent_item_boundaries_mixed_expansions(split):
    """The persistent grid's item boundaries -- the next item's first tiles issued while
    the current one finishes, its run parameters copied ahead -- over items of every
    shape: LO runs with no tiles at all, windows of 3 and 5 steps with fewer tiles than
    the stage ring holds, classical and quantum NLO runs, 427 chunk items for 152 CTAs
    (several per CTA, the run changing between them or not). Bitwise the same as one CTA
    per item: n, omega, c, E and rows of F and rho."""
    from kb2pi import capi

    cfgs = [dict(Ns=40, M=33, lam=2.0, T=1.0, pexp=1), dict(Ns=32, M=3, lam=3.0, T=1.5, pexp=2),
            dict(Ns=24, M=64, lam=1.0, T=0.7, pexp=0), dict(Ns=16, M=5, lam=4.0, T=2.0, pexp=1),
            dict(Ns=8, M=100, lam=2.0, T=1.2, pexp=1)]
    out = []
    for pers in (0, 1):
        ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=c["pexp"], precision=1, device=0, flags=0,
                            dt=0.1, lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
        h = capi.Handle(ps)
        for r, c in enumerate(cfgs):
            _, k2, _ = h.orbits(r)
            h.init(r, occupation(dict(c), k2), 1.0)
        h.set_tuning(memint_variant=2, memint_split=split, batch_order=1, memint_persistent=pers)
        h.steps(3, 110, 0)
        rows = []
        for r in range(len(cfgs)):
            tmin, _ = h.window(r)
            rows.append((h.measure(r, 112), [(h.get(r, 0, 112, tp), h.get(r, 1, 112, tp)) for tp in (tmin, 111, 112)]))
        out.append(rows)
        h.close()
    for (ma, ra), (mb, rb) in zip(out[0], out[1]):
        assert ma["E"] == mb["E"] and ma["M2"] == mb["M2"]
        for k in ("n", "omega", "c", "F", "ddF"):
            assert np.array_equal(ma[k], mb[k]), k
        for (Fa, Ra), (Fb, Rb) in zip(ra, rb):
            assert np.array_equal(Fa, Fb) and np.array_equal(Ra, Rb)


@pytest.mark.parametrize("precision,variant,persistent", [(0, None, 0), (1, None, 0), (1, 2, 0), (0, None, 1),
                                                          (1, 2, 1)])
def test_bounded_wait_runs_out_and_is_reported(precision, variant, persistent):
    """Failure detection without a GPU fault: with the test hook the memory-
    integral producer issues no tiles, so every consumer's bounded wait runs out
    (about 2 s), the kernel sets its error bit, frees its tensor memory and
    returns; kb_sync reports KB_ERR_TIMEOUT once and the device keeps working
    (a new handle evolves and measures)."""
    from kb2pi import capi

    cfg = dict(Ns=6, M=8, N=4, lam=2.0, dt=0.1, pexp=1, T=1.5)
    h = make_gpu(cfg, precision)
    _, k2, _ = h.orbits()
    h.init(0, occupation(cfg, k2), 1.0)
    if variant is not None:  # the leapfrog warps leave their hand-off wait when the consumers abort
        h.set_tuning(memint_variant=variant)
    if persistent:  # an aborted item ends its CTA's queue loop
        h.set_tuning(memint_persistent=1)
    h.steps(3, 5, 0)
    h.sync()
    h.set_tuning(test_no_tiles=1)
    t0 = time.time()
    h.step(8)
    with pytest.raises(capi.KbError, match="KB_ERR_TIMEOUT"):
        h.sync()
    assert time.time() - t0 < 60
    h.set_tuning(test_no_tiles=0)  # synchronises: the error was reported once and cleared
    h.close()
    g = make_gpu(cfg, precision)
    g.init(0, occupation(cfg, k2), 1.0)
    g.steps(3, 20, 0)
    m = g.measure(0, 22)
    assert np.isfinite(m["E"]) and np.all(np.isfinite(m["n"]))
    g.close()



@pytest.mark.parametrize("precision", [0, 1])
def test_pipelined_timeout_is_reported_once(precision):
    """The measurement loop one step behind (kb_measure_enqueue / kb_measure_take):
    step t times out (test hook: no tiles issued), step t+1 is issued before t is
    taken. The enqueue of t clears the device flags in stream order right after
    copying them, so the synchronising kb_set_tuning between the two steps sees a
    clean flag, the take of t reports KB_ERR_TIMEOUT and nothing reports it again."""
    from kb2pi import capi

    cfg = dict(Ns=6, M=8, N=4, lam=2.0, dt=0.1, pexp=1, T=1.5)
    h = make_gpu(cfg, precision)
    _, k2, _ = h.orbits()
    h.init(0, occupation(cfg, k2), 1.0)
    h.steps(3, 5, 0)
    h.sync()
    h.set_tuning(test_no_tiles=1)
    t0 = time.time()
    h.step(8)
    h.measure_enqueue(0, 8)
    h.set_tuning(test_no_tiles=0)  # waits for step 8; its flag was cleared behind the copy
    h.step(9)
    h.measure_enqueue(0, 9)
    timeouts = 0
    for call in (lambda: h.measure_take(0, 8), lambda: h.measure_take(0, 9), h.sync):
        try:
            call()
        except capi.KbError as e:
            if "KB_ERR_TIMEOUT" in str(e):
                timeouts += 1
    assert timeouts == 1
    assert time.time() - t0 < 60
    h.close()


@pytest.mark.parametrize("precision,split,pers", [(0, 0, 0), (1, 0, 0), (1, 2, 0), (0, 0, 1), (1, 2, 1)])
def test_batch_overlap_is_bitwise_the_one_launch_step(precision, split, pers):
    """Concurrent groups (batch_overlap: the second group's sunset on its own stream
    beside the first group's memory integrals; with the persistent grid, the first
    group's memory integrals on the SMs the sunset leaves free) change which launch
    computes a run, not how: every run is bitwise the same as with one launch per
    kernel, through kb_step and the captured graph of kb_steps alike."""
    from kb2pi import capi

    cfgs = [dict(Ns=8, M=20, lam=2.0, T=1.0), dict(Ns=16, M=45, lam=4.0, T=2.0), dict(Ns=12, M=33, lam=1.0, T=0.7),
            dict(Ns=6, M=9, lam=3.0, T=1.5), dict(Ns=10, M=27, lam=2.5, T=1.2)]
    out = []
    for ov in (0, 20, 76):
        ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=precision, device=0, flags=0,
                            dt=0.1, lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
        h = capi.Handle(ps)
        for r, c in enumerate(cfgs):
            _, k2, _ = h.orbits(r)
            h.init(r, occupation(dict(c), k2), 1.0)
        h.set_tuning(batch_overlap=ov, memint_split=split, memint_persistent=pers)
        assert h.tuning()["batch_overlap"] == ov and h.tuning()["memint_persistent"] == pers
        h.steps(3, 30, 0)
        for t in range(33, 41):
            h.step(t)
        out.append([(h.measure(r, 40), h.get(r, 0, 40, 37)) for r in range(len(cfgs))])
        h.close()
    for o in out[1:]:
        for (ma, ra), (mb, rb) in zip(out[0], o):
            assert ma["E"] == mb["E"] and np.array_equal(ma["n"], mb["n"]) and np.array_equal(ra, rb)


def test_batch_overlap_errors_and_autotune():
    from kb2pi import capi

    h = make_gpu(CFG, 1)
    with pytest.raises(capi.KbError, match="batch_overlap"):
        h.set_tuning(batch_overlap=10)  # one run: nothing to overlap
    h.close()
    cfgs = [dict(Ns=8, M=20, lam=2.0, T=1.0), dict(Ns=12, M=30, lam=3.0, T=1.5)]
    ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=1, device=0, flags=0, dt=0.1,
                        lam=c["lam"], mass2=1.0, mass=1.0) for c in cfgs]
    h = capi.Handle(ps)
    for r, c in enumerate(cfgs):
        _, k2, _ = h.orbits(r)
        h.init(r, occupation(dict(c), k2), 1.0)
    h.steps(3, 25, 0)
    d = h.autotune(trials=1)
    assert d["batch_overlap"] >= 0
    m = [h.measure(r, 27)["E"] for r in range(2)]
    assert all(np.isfinite(m))
    with pytest.raises(capi.KbError, match="batch_overlap"):
        h.set_tuning(batch_overlap=10 ** 6)
    h.close()
