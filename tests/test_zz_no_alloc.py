"""kb_sunset_rows_noalloc: the self-energy entry point that allocates nothing.

It serves callers that cannot call cudaMalloc themselves (their device memory
belongs to their own pool, or an allocation must not synchronise the device),
so its scratch is a fixed device array inside the library. This file is
collected last: if it fails, a run that stops at the first failure has
already run every other test. It passes alone in a fresh process too: the
entry point's first call on a device does its own set-up.
"""
import ctypes

import numpy as np
import pytest

from kbtest_util import make_gpu, make_oracle, occupation, random_symmetric_row, rel


def _lib():
    from kb2pi import capi

    return capi.load_library()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib()
    rc = lib.kb_sunset_rows_noalloc(48, 4, 1.0, 1, 3, None, None, None, None, None)
    assert rc == -1
    assert b"Ns=48" in lib.kb_last_error(None)


@pytest.mark.gpu
@pytest.mark.parametrize("Ns,nrows,pexp", [
    (16, 10, 1),    # LambdaNLO quantum
    (32, 300, 1),   # the largest Ns the fixed scratch takes; more rows than SMs, so a CTA reuses its slot
    (12, 40, 2),    # LambdaNLO classical
])
def test_noalloc_matches_kb_self_energies_twice(Ns, nrows, pexp):
    """Two calls in a row through the C ABI, each checked against the handle path
    (kb_self_energies + kb_get_sigma) on the same rows, FP64 tolerance 1e-12."""
    import torch

    lib = _lib()
    N, lam = 8, 10.0
    tmone = nrows
    cfg = dict(Ns=Ns, M=nrows + 4, dt=0.01, lam=lam, N=N, T=2.0, pexp=pexp)
    g = make_gpu(cfg)  # KB_PREC_FP64: the same sunset as the no-alloc variant
    oracle = make_oracle(cfg)
    _, k2, _ = g.orbits(0)
    g.init(0, occupation(cfg, k2), 1.0)
    for t in range(3, 11):
        g.step(t)
    for _ in range(11, tmone + 2):  # the window [1, tmone + 1], rows overwritten below
        g.expand()
    S = g.S[0]
    stream = torch.cuda.current_stream()
    for call, seed in enumerate((11, 22)):
        rng = np.random.default_rng(seed + Ns + pexp)
        Frows = np.zeros((tmone, S))
        rrows = np.zeros((tmone, S))
        for i, tp in enumerate(range(1, tmone + 1)):
            Frows[i] = random_symmetric_row(S, rng)
            rrows[i] = 0.0 if tp == tmone else random_symmetric_row(S, rng)
            g.set(0, 0, tmone, tp, Frows[i])
            g.set(0, 1, tmone, tp, rrows[i])
        g.self_energies(tmone)
        ref_F = np.array([g.sigma(0, 0, tp) for tp in range(1, tmone + 1)])
        ref_r = np.array([g.sigma(0, 1, tp) for tp in range(1, tmone + 1)])

        dF = torch.tensor(Frows, dtype=torch.float64, device="cuda")
        dr = torch.tensor(rrows, dtype=torch.float64, device="cuda")
        oF = torch.full((tmone, S), float("nan"), dtype=torch.float64, device="cuda")
        orr = torch.full((tmone, S), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.kb_sunset_rows_noalloc(Ns, N, lam, pexp, tmone, ctypes.c_void_p(dF.data_ptr()),
                                        ctypes.c_void_p(dr.data_ptr()), ctypes.c_void_p(oF.data_ptr()),
                                        ctypes.c_void_p(orr.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.kb_last_error(None)
        stream.synchronize()
        gotF, gotr = oF.cpu().numpy(), orr.cpu().numpy()
        assert np.all(np.isfinite(gotF)) and np.all(np.isfinite(gotr)), call
        assert rel(gotF, ref_F) <= 1e-12, call
        assert rel(gotr, ref_r) <= 1e-12, call
        # and directly against the CPU FP64 oracle's sunset on a few of the same rows
        for i in (0, tmone // 2, tmone - 1):
            oF, orr = oracle.sunset_rows(Frows[i], rrows[i])
            assert rel(gotF[i], oF) <= 1e-12, (call, i)
            assert rel(gotr[i], orr) <= 1e-12 or np.max(np.abs(orr)) == 0.0, (call, i)
    g.close()
    oracle.close()
