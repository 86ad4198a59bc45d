"""Shared helpers of the parity tests: seeded inputs and GPU/oracle drivers."""
from __future__ import annotations

import numpy as np

from oracle import ENGINE_FULL, ENGINE_OCTANT, ENGINE_ORBIT, Oracle  # noqa: F401

PEXP_NAMES = {0: "LambdaLO", 1: "LambdaNLO", 2: "LambdaNLOclassical"}


def thermal_n(k2, T, mass=1.0):
    """getparticlenr(::TwoPIScalarThermal) (TwoPIScalar_Initialization.jl:138-140)."""
    return 1.0 / (np.exp(np.sqrt(np.asarray(k2) + mass ** 2) / (T * mass)) - 1.0)


def tsunami_n(k2):
    return 5.0 * np.exp(-((np.sqrt(np.asarray(k2)) - 1.0) ** 2) / (2 * 0.2 ** 2))


def random_symmetric_row(S, rng):
    """createrandomF (Tests/TwoPIScalar_Tests_LambdaNLO_checkfastimplementation.jl:5-16):
    one value rand() - 0.5 per orbit, here from a seeded generator."""
    return rng.random(S) - 0.5


def make_gpu(cfg, precision=0, device=0):
    from kb2pi import capi

    p = capi.KbParams(Ns=cfg["Ns"], sdim=3, M=cfg["M"], N=cfg.get("N", 4), pexp=cfg.get("pexp", 1),
                      precision=precision, device=device, flags=cfg.get("flags", 0), dt=cfg["dt"], lam=cfg["lam"],
                      mass2=cfg.get("mass2", 1.0), mass=cfg.get("mass", 1.0))
    return capi.Handle([p])


def make_oracle(cfg, engine=ENGINE_OCTANT, nthreads=4):
    return Oracle(cfg["Ns"], 3, M=cfg["M"], N=cfg.get("N", 4), dt=cfg["dt"], lam=cfg["lam"],
                  mass2=cfg.get("mass2", 1.0), mass=cfg.get("mass", 1.0), pexp=cfg.get("pexp", 1),
                  engine=engine, nthreads=nthreads)


def occupation(cfg, k2):
    if cfg.get("init", "thermal") == "thermal":
        return thermal_n(k2, cfg.get("T", 2.0), cfg.get("mass", 1.0))
    return tsunami_n(k2)


def rel(a, b):
    """max |a - b| / max |b| (normalised so zeros of rho do not blow up)."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    den = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / den)
