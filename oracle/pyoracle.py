"""ctypes binding of libkb_oracle.so (the CPU FP64 restatement in kb_oracle.cpp).

Test infrastructure: the oracle the CUDA path is compared against. Parity of
this oracle with the Julia reference itself is unpinned (no Julia here); see
kb_oracle.h for what pins it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

ENGINE_FULL, ENGINE_ORBIT, ENGINE_OCTANT = 0, 1, 2
PEXP_LO, PEXP_NLO_QUANTUM, PEXP_NLO_CLASSICAL, PEXP_NINV_LO, PEXP_NINV_NLO = 0, 1, 2, 3, 4

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_LOCK = threading.Lock()


class OracleParams(C.Structure):
    _fields_ = [
        ("Ns", C.c_int32), ("sdim", C.c_int32), ("M", C.c_int32), ("N", C.c_int32),
        ("pexp", C.c_int32), ("engine", C.c_int32), ("nthreads", C.c_int32), ("pad_", C.c_int32),
        ("dt", C.c_double), ("lam", C.c_double), ("mass2", C.c_double), ("mass", C.c_double),
    ]


class OracleScalars(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")]


def build_oracle(force: bool = False) -> str:
    """Compile oracle/libkb_oracle.so with the committed Makefile."""
    so = os.path.join(_HERE, "libkb_oracle.so")
    src = os.path.join(_HERE, "kb_oracle.cpp")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "libkb_oracle.so"], check=True)
    return so


def _lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            lib = C.CDLL(build_oracle())
            P = C.POINTER
            d, i32, i64 = C.c_double, C.c_int32, C.c_int64
            lib.orc_create.restype = C.c_void_p
            lib.orc_create.argtypes = [P(OracleParams)]
            lib.orc_destroy.argtypes = [C.c_void_p]
            lib.orc_num_orbits.argtypes = [C.c_void_p]
            lib.orc_num_sites.argtypes = [C.c_void_p]
            lib.orc_num_sites.restype = i64
            lib.orc_orbits.argtypes = [C.c_void_p, P(i32), P(d), P(i64)]
            lib.orc_site_orbit.argtypes = [C.c_void_p, P(i32)]
            lib.orc_init_occupation.argtypes = [C.c_void_p, P(d), d]
            lib.orc_init_gauss.argtypes = [C.c_void_p, d, d, d]
            lib.orc_step.argtypes = [C.c_void_p, i32]
            lib.orc_expand.argtypes = [C.c_void_p]
            lib.orc_self_energies.argtypes = [C.c_void_p, i32]
            lib.orc_measure.argtypes = [C.c_void_p, i32, P(OracleScalars)] + [P(d)] * 9
            lib.orc_get.argtypes = [C.c_void_p, i32, i32, i32, P(d)]
            lib.orc_set.argtypes = [C.c_void_p, i32, i32, i32, P(d)]
            lib.orc_get_sigma.argtypes = [C.c_void_p, i32, i32, P(d)]
            lib.orc_get_lattice.argtypes = [C.c_void_p, i32, i32, i32, P(d)]
            lib.orc_window.argtypes = [C.c_void_p, P(i32), P(i32)]
            lib.orc_hartree_mass2.argtypes = [C.c_void_p, i32, i32]
            lib.orc_hartree_mass2.restype = d
            lib.orc_hartree_prefactor.argtypes = [C.c_void_p]
            lib.orc_hartree_prefactor.restype = d
            lib.orc_gap_mass.argtypes = [C.c_void_p, P(d), d]
            lib.orc_gap_mass.restype = d
            lib.orc_sunset_rows.argtypes = [C.c_void_p, P(d), P(d), P(d), P(d)]
            lib.orc_step_times.argtypes = [C.c_void_p, P(d), P(d)]
            lib.orc_dual_loss.argtypes = [P(OracleParams), P(d), d, i32, P(d), d, P(d), P(d), P(d)]
            _LIB = lib
    return _LIB


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with code {rc}")


def dual_loss(Ns, M, n_init, init_mass, t_final, w_n=None, w_E=0.0, dn=None, N=4, dt=0.1, lam=1.0, mass2=1.0,
              mass=1.0, pexp=PEXP_NLO_QUANTUM):
    """Forward-mode (dual-number) derivatives of L = sum w_n n(t_final) + w_E E(t_final):
    returns (L, dL/dlambda, dL/dm^2, dL/dn_init . dn) from the templated orbit/octant engine."""
    lib = _lib()
    p = OracleParams(Ns=Ns, sdim=3, M=M, N=N, pexp=pexp, engine=ENGINE_OCTANT, nthreads=1, pad_=0, dt=dt,
                     lam=lam, mass2=mass2, mass=mass)
    n0 = np.ascontiguousarray(n_init, dtype=np.float64)
    wn = None if w_n is None else np.ascontiguousarray(w_n, dtype=np.float64)
    d = None if dn is None else np.ascontiguousarray(dn, dtype=np.float64)
    L = C.c_double()
    dL = np.zeros(3)
    _check(lib.orc_dual_loss(C.byref(p), _dp(n0), float(init_mass), int(t_final), _dp(wn), float(w_E), _dp(d),
                             C.byref(L), _dp(dL)), "dual_loss")
    return L.value, dL[0], dL[1], dL[2]


class Oracle:
    """One simulation on the CPU oracle; mirrors QFTdynamicsSolution for TwoPIScalar."""

    def __init__(self, Ns, sdim=3, M=10, N=4, dt=0.1, lam=1.0, mass2=1.0, mass=1.0,
                 pexp=PEXP_NLO_QUANTUM, engine=ENGINE_OCTANT, nthreads=1):
        self.lib = _lib()
        self.p = OracleParams(Ns=Ns, sdim=sdim, M=M, N=N, pexp=pexp, engine=engine,
                              nthreads=nthreads, pad_=0, dt=dt, lam=lam, mass2=mass2, mass=mass)
        self.h = self.lib.orc_create(C.byref(self.p))
        if not self.h:
            raise ValueError("oracle rejected the parameters")
        self.S = self.lib.orc_num_orbits(self.h)
        self.V = self.lib.orc_num_sites(self.h)
        self.M = M
        self.dt = dt

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    # --- orbit tables -----------------------------------------------------
    def orbits(self):
        rep = np.zeros((self.S, 3), np.int32)
        k2 = np.zeros(self.S)
        deg = np.zeros(self.S, np.int64)
        self.lib.orc_orbits(self.h, rep.ctypes.data_as(C.POINTER(C.c_int32)), _dp(k2),
                            deg.ctypes.data_as(C.POINTER(C.c_int64)))
        return rep, k2, deg

    def site_orbit(self):
        out = np.zeros(self.V, np.int32)
        self.lib.orc_site_orbit(self.h, out.ctypes.data_as(C.POINTER(C.c_int32)))
        return out

    # --- dynamics ---------------------------------------------------------
    def init_occupation(self, n, init_mass):
        n = np.ascontiguousarray(n, dtype=np.float64)
        _check(self.lib.orc_init_occupation(self.h, _dp(n), float(init_mass)), "init")

    def init_gauss(self, xi, eta, sig):
        _check(self.lib.orc_init_gauss(self.h, xi, eta, sig), "init_gauss")

    def step(self, t):
        _check(self.lib.orc_step(self.h, int(t)), f"step({t})")

    def expand(self):
        _check(self.lib.orc_expand(self.h), "expand")

    def self_energies(self, tmone):
        _check(self.lib.orc_self_energies(self.h, int(tmone)), "self_energies")

    def window(self):
        a, b = C.c_int32(), C.c_int32()
        self.lib.orc_window(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def get(self, which, a, b):
        out = np.zeros(self.S)
        _check(self.lib.orc_get(self.h, which, a, b, _dp(out)), f"get({which},{a},{b})")
        return out

    def set(self, which, a, b, vals):
        v = np.ascontiguousarray(vals, dtype=np.float64)
        _check(self.lib.orc_set(self.h, which, a, b, _dp(v)), "set")

    def F(self, a, b):
        return self.get(0, a, b)

    def rho(self, a, b):
        return self.get(1, a, b)

    def sigma(self, which, z):
        out = np.zeros(self.S)
        _check(self.lib.orc_get_sigma(self.h, which, z, _dp(out)), "sigma")
        return out

    def lattice(self, which, a, b):
        out = np.zeros(self.V)
        _check(self.lib.orc_get_lattice(self.h, which, a, b, _dp(out)), "lattice")
        return out

    def step_times(self):
        a, b = C.c_double(), C.c_double()
        self.lib.orc_step_times(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def hartree_mass2(self, a, b):
        return self.lib.orc_hartree_mass2(self.h, a, b)

    def hartree_prefactor(self):
        return self.lib.orc_hartree_prefactor(self.h)

    def gap_mass(self, n, x0=0.5):
        n = np.ascontiguousarray(n, dtype=np.float64)
        return self.lib.orc_gap_mass(self.h, _dp(n), float(x0))

    def sunset_rows(self, F, rho):
        F = np.ascontiguousarray(F, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        sF, sr = np.zeros(self.S), np.zeros(self.S)
        _check(self.lib.orc_sunset_rows(self.h, _dp(F), _dp(rho), _dp(sF), _dp(sr)), "sunset")
        return sF, sr

    def measure(self, t):
        sc = OracleScalars()
        arrs = {k: np.zeros(self.S) for k in ("F", "ddF", "n", "omega", "c")}
        tr = {k: np.zeros(self.M) for k in ("Fonet", "ronet", "SigF", "Sigr")}
        _check(self.lib.orc_measure(self.h, int(t), C.byref(sc), _dp(arrs["F"]), _dp(arrs["ddF"]),
                                    _dp(arrs["n"]), _dp(arrs["omega"]), _dp(arrs["c"]),
                                    _dp(tr["Fonet"]), _dp(tr["ronet"]), _dp(tr["SigF"]),
                                    _dp(tr["Sigr"])), f"measure({t})")
        out = {k: getattr(sc, k) for k in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")}
        out.update(arrs)
        tmin, tmax = self.window()
        nw = tmax - tmin
        for k, v in tr.items():
            out[k] = v[:nw].copy()
        return out
