"""The KB_DEBUG build (libkb2pi_debug.so): device-side bounds checks on ring,
tile and Sigma indices stay clear on small lattices and windows (Ns = 4..8,
M = 3..10, wrapping rings, both precisions, every memory-integral split mode,
the persistent memory-integral grid, a batch of uneven runs), and the checked build computes what the release build
computes. The checked library runs in a child process (KB2PI_LIB selects it for
that process); a failed check would surface as KB_ERR_RANGE from kb_sync.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DEBUG_LIB = os.path.join(ROOT, "qftdynamicsm.jl_gb300", "kb2pi", "libkb2pi_debug.so")

CASES = [
    # (runs, precision, memint_split[, sunset_variant[, memint_persistent]]): each run (Ns, M, lambda, T)
    ([(4, 3, 2.0, 1.5)], 0, 0),
    ([(8, 9, 2.0, 1.5), (6, 5, 3.0, 2.0)], 1, 0, 2),  # the tensor-core sunset
    ([(6, 5, 3.0, 2.0)], 0, 1),
    ([(8, 10, 2.0, 1.0)], 1, 0),
    ([(8, 7, 4.0, 2.0)], 1, 1),
    ([(8, 9, 1.0, 1.5)], 1, 2),
    ([(4, 3, 2.0, 1.5), (6, 10, 3.0, 1.0), (8, 6, 1.5, 2.5)], 1, 2),
    ([(6, 4, 2.0, 1.5), (8, 9, 3.0, 2.0)], 0, 2),
    ([(4, 3, 2.0, 1.5), (6, 10, 3.0, 1.0), (8, 6, 1.5, 2.5)], 1, 2, 0, 1),  # persistent memory integrals
    ([(6, 4, 2.0, 1.5), (8, 9, 3.0, 2.0)], 0, 1, 0, 1),
]
STEPS = 24


def run_cases():
    """Every case for STEPS steps on the library of this process; per case and run
    the final E and n and one F row, as lists."""
    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.join(ROOT, "qftdynamicsm.jl_gb300"))
    from kb2pi import capi

    out = []
    for runs, prec, split, *sv in CASES:
        ps = [capi.KbParams(Ns=Ns, sdim=3, M=M, N=4, pexp=1, precision=prec, device=0, flags=0, dt=0.1, lam=lam,
                            mass2=1.0, mass=1.0) for Ns, M, lam, _ in runs]
        h = capi.Handle(ps)
        for r, (_, _, _, T) in enumerate(runs):
            _, k2, _ = h.orbits(r)
            h.init(r, 1.0 / (np.exp(np.sqrt(k2 + 1.0) / T) - 1.0), 1.0)
        if sv:
            h.set_tuning(sunset_variant=sv[0])
        if len(sv) > 1:
            h.set_tuning(memint_persistent=sv[1])
        h.steps(3, 4, 0)
        if split and prec == 1:
            h.set_tuning(memint_variant=2 if split == 2 else 1, memint_split=split)
        elif split:
            h.set_tuning(memint_split=split)
        for t in range(7, 3 + STEPS):
            h.step(t)
        h.sync()  # raises KB_ERR_RANGE if a device bounds check failed
        t = 2 + STEPS
        res = []
        for r in range(len(runs)):
            m = h.measure(r, t)
            res.append({"E": m["E"], "n": m["n"].tolist(), "F": h.get(r, 0, t, t - 2).tolist()})
        out.append(res)
        h.close()
    return out


@pytest.mark.gpu
def test_debug_build_checks_stay_clear_and_match_release():
    if not os.path.exists(DEBUG_LIB):
        pytest.fail(f"{DEBUG_LIB} is missing: __graft_entry__.build() builds it")
    env = dict(os.environ, KB2PI_LIB=DEBUG_LIB)
    p = subprocess.run([sys.executable, os.path.abspath(__file__), "--child"], env=env, capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-3000:]
    dbg = json.loads(p.stdout.strip().splitlines()[-1])
    rel = run_cases()
    assert len(dbg) == len(rel) == len(CASES)
    for case, (a, b) in enumerate(zip(dbg, rel)):
        for r, (x, y) in enumerate(zip(a, b)):
            assert abs(x["E"] - y["E"]) <= 1e-13 * abs(y["E"]), (case, r)
            assert np.max(np.abs(np.array(x["n"]) - y["n"])) <= 1e-13 * np.max(np.abs(y["n"])), (case, r)
            assert np.max(np.abs(np.array(x["F"]) - y["F"])) <= 1e-13 * np.max(np.abs(y["F"])), (case, r)


if __name__ == "__main__" and "--child" in sys.argv:
    print(json.dumps(run_cases()))
