"""The C-ABI library loads and exports every symbol include/kb2pi.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kb2pi.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(kb_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_binding_list():
    from kb2pi import capi

    assert sorted(capi.EXPORTS) == declared_symbols()


def test_julia_glue_calls_declared_symbols_only():
    """julia/TwoPIScalar_GPU.jl (not executed here: no Julia) and the bindings shown in
    INTEGRATION.md name only functions the header declares, with as many arguments in
    each Julia ccall as the C declaration has parameters."""
    declared = set(declared_symbols())
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    arity = {}
    for name, params in re.findall(r"\b(kb_[a-z_0-9]+)\s*\(([^)]*)\)\s*;", src):
        params = params.strip()
        arity[name] = 0 if params in ("", "void") else params.count(",") + 1
    jl = open(os.path.join(ROOT, "qftdynamicsm.jl_gb300", "julia", "TwoPIScalar_GPU.jl")).read()
    calls = re.findall(r"ccall\(\(:(kb_[a-z_0-9]+)\s*,[^)]*\)\s*,\s*[A-Za-z_{}0-9]+\s*,\s*\(([^)]*)\)", jl)
    assert calls
    for name, types in calls:
        assert name in declared, name
        n = len([x for x in types.split(",") if x.strip()])
        assert n == arity[name], (name, n, arity[name])
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    for name in set(re.findall(r"\b(kb_[a-z_0-9]+)\(", doc)):
        assert name in declared, name


def test_library_exports_all_symbols():
    from kb2pi import capi

    lib = capi.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
        assert ctypes.cast(getattr(lib, name), ctypes.c_void_p).value


def test_debug_library_exports_all_symbols():
    """libkb2pi_debug.so (the KB_DEBUG build with device-side bounds checks) is built
    by __graft_entry__.build() next to the release library and has the same ABI."""
    path = os.path.join(ROOT, "qftdynamicsm.jl_gb300", "kb2pi", "libkb2pi_debug.so")
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert ctypes.cast(getattr(lib, name), ctypes.c_void_p).value, name


def test_create_rejects_bad_parameters_without_touching_a_gpu():
    from kb2pi import capi

    lib = capi.load_library()
    h = ctypes.c_void_p()
    p = capi.KbParams(Ns=7, sdim=3, M=10, N=4, pexp=1, precision=0, device=0, flags=0, dt=0.1, lam=1.0,
                      mass2=1.0, mass=1.0)
    assert lib.kb_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert b"Ns=7" in lib.kb_last_error(None)
    p.Ns, p.M = 8, 2
    assert lib.kb_create(ctypes.byref(p), ctypes.byref(h)) == -1
    p.M, p.sdim = 10, 2
    assert lib.kb_create(ctypes.byref(p), ctypes.byref(h)) == -1


def test_create_without_device_fails_loudly():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    from kb2pi import capi

    p = capi.KbParams(Ns=8, sdim=3, M=10, N=4, pexp=1, precision=0, device=0, flags=0, dt=0.1, lam=1.0,
                      mass2=1.0, mass=1.0)
    with pytest.raises(capi.KbError) as ei:
        capi.Handle([p])
    assert ei.value.code in (-7, -3)


def test_julia_glue_covers_the_initial_states_of_the_mirror():
    """Every initial state the Python mirror initialises on the lattice has its
    occupation in the Julia glue (getparticlenr_orbits), and the Gauss state goes
    through kb_init_rows, as in the mirror (TwoPIScalar_Initialization.jl:95-203)."""
    jl = open(os.path.join(ROOT, "qftdynamicsm.jl_gb300", "julia", "TwoPIScalar_GPU.jl")).read()
    have = set(re.findall(r"getparticlenr_orbits\(init::TwoPIScalar(\w+),", jl))
    assert {"Particle", "Thermal", "Tsunami", "Quench", "TopHatT1", "TopHatT2", "TopHatT3"} <= have
    gauss = jl[jl.index("if init isa TwoPIScalarGauss"):]
    gauss = gauss[:gauss.index("else")]
    assert ":kb_init_rows" in gauss
    # the TopHat ranges and heights are the mirror's (lo, hi, eta)
    from kb2pi import twopiscalar  # noqa: F401
    for name, lo, hi, eta in (("T1", "0.68", "2.04", "2"), ("T2", "0.0", "1.9", "1.85"), ("T3", "2.04", "2.72", "1.6")):
        assert f"TwoPIScalarTopHat{name}, disc, k2s) = tophat_orbits(disc, k2s, {lo}, {hi}, {eta})" in jl
