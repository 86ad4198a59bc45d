"""Host side of the Python mirror of the reference's problem setup, without a GPU:
cubic orbits of the lattice (the numbering libkb2pi and the oracle share),
check_parameters! (src/DefAbstractSimSetup.jl:21-31), QFTdynamicsProblem with
Renormalize (TwoPIScalar_ModelExpansionRenormalization.jl:18-47) and the
occupation profiles of getparticlenr (TwoPIScalar_Initialization.jl:133-203)."""
import math

import numpy as np
import pytest

from oracle import Oracle


def _params(**kw):
    p = dict(Nx=8, sdim=3, Mass=1.0, Nsteps=40, dt=0.1, NstepsinMemory=0, Nmeas=0, Lambda=2.0, ONgroup=4,
             init="Thermal", T=2.0, Pexp="LambdaNLO", Reno="RNone", Num="GPU")
    p.update(kw)
    return p


@pytest.mark.parametrize("Ns", [2, 4, 8, 12])
def test_lattice_orbits_match_the_oracle(Ns):
    from kb2pi.twopiscalar import lattice_orbits

    reps, k2, deg = lattice_orbits(Ns)
    o = Oracle(Ns, 3, M=4, N=4, lam=1.0, mass2=1.0)
    _, k2o, dego = o.orbits()
    o.close()
    assert np.allclose(k2, k2o, rtol=0, atol=1e-13)
    assert np.array_equal(deg, np.asarray(dego, np.int64))
    assert deg.sum() == Ns ** 3  # every site in exactly one orbit
    assert len(reps) == math.comb(Ns // 2 + 3, 3)
    assert np.all(reps[:, 0] <= reps[:, 1]) and np.all(reps[:, 1] <= reps[:, 2])


def test_check_parameters_defaults():
    from kb2pi.twopiscalar import check_parameters

    p = _params(Nsteps=40, NstepsinMemory=0, Nmeas=0)
    check_parameters(p)
    assert p["NstepsinMemory"] == 42 and p["Nmeas"] == 40
    p = _params(Nsteps=40, NstepsinMemory=10, Nmeas=8)
    check_parameters(p)
    assert p["NstepsinMemory"] == 10 and p["Nmeas"] == 8


@pytest.mark.parametrize("mod,pexp", [("phi4", "LambdaNLO"), ("phi4tachyonic", "LambdaNLO"),
                                      ("phi4", "NinverseLO")])
def test_problem_with_mass_renormalisation(mod, pexp):
    from kb2pi.twopiscalar import TwoPIScalarfile, lattice_orbits, make_problem

    p = _params(Mod=mod, Pexp=pexp, Reno="RMass", Nsteps=40, Nmeas=10)
    prob = make_problem(TwoPIScalarfile(), p)
    assert prob.disc.Nx == 8 and prob.disc.vol == 512 and prob.disc.NstepsinMemory == 42
    assert prob.simsetup.NstepsbetweenNmeas == 4 and prob.simsetup.Nsteps == 40
    # counterterm: -(Hartree prefactor) ivol sum_k deg_k / (2 omega_k), omega_k = sqrt(k^2 + m^2)
    _, k2, deg = lattice_orbits(8)
    pref = 2.0 / 6 if pexp == "NinverseLO" else 2.0 * 6 / 24
    ct = -pref / 512 * float(np.sum(deg / (2 * np.sqrt(k2 + 1.0))))
    want = (-1.0 if mod == "phi4tachyonic" else 1.0) + ct
    assert abs(prob.model.Mass2 - want) <= 1e-14
    assert prob.model.tachyonic == (mod == "phi4tachyonic")
    plain = make_problem(TwoPIScalarfile(), _params(Mod=mod, Pexp=pexp, Reno="RNone"))
    assert plain.model.Mass2 == 1.0


def test_problem_rejects_what_the_gpu_numerics_do_not_run():
    from kb2pi.twopiscalar import TwoPIScalarfile, make_problem

    with pytest.raises(ValueError, match="Pexp"):
        make_problem(TwoPIScalarfile(), _params(Pexp="NoSuchExpansion"))
    with pytest.raises(ValueError, match="Num"):
        make_problem(TwoPIScalarfile(), _params(Num="CPUfull"))
    with pytest.raises(ValueError, match="renormalisation"):
        make_problem(TwoPIScalarfile(), _params(Reno="RSomething"))


def test_occupation_profiles():
    from kb2pi.twopiscalar import Discretization, Init, getparticlenr, lattice_orbits

    _, k2, _ = lattice_orbits(16)
    disc = Discretization(1.0, 16, 3, 10, 0.1, 16 ** 3, 1 / 16 ** 3, 12, 10)
    th = getparticlenr(Init("Thermal", T=2.0), disc, k2)
    assert np.allclose(th, 1.0 / (np.exp(np.sqrt(k2 + 1.0) / 2.0) - 1.0), rtol=1e-15)
    assert np.all(getparticlenr(Init("Pnr", n=3.0), disc, k2) == 3.0)
    assert np.all(getparticlenr(Init("Quench"), disc, k2) == 0.0)
    ts = getparticlenr(Init("Tsunami"), disc, k2)
    assert np.allclose(ts, 5.0 * np.exp(-((np.sqrt(k2) - 1.0) ** 2) / 0.08), rtol=1e-15)
    # TopHatT1: eta = 2 on the lev2 levels between the ones closest to 0.68 and 2.04 x sdim m^2
    th1 = getparticlenr(Init("TopHatT1"), disc, k2)
    levels = np.unique(k2)
    lo = levels[np.argmin(np.abs(levels - 0.68 * 3))]
    hi = levels[np.argmin(np.abs(levels - 2.04 * 3))]
    inside = (k2 >= lo) & (k2 <= hi)
    assert inside.any() and (~inside).any()
    assert np.all(th1[inside] == 2.0) and np.all(th1[~inside] == 0.0)
    with pytest.raises(ValueError):
        getparticlenr(Init("NoSuchInit"), disc, k2)


def test_orbits_to_shells_groups_equal_lev2():
    """Per-orbit arrays onto lev2 shells: the shell value is the site average, and at
    Ns=4 the orbits (0,1,1) and (0,0,2) share lev2 = 4 and so one shell."""
    from kb2pi.twopiscalar import lattice_orbits, orbits_to_shells

    rep, k2, deg = lattice_orbits(4)
    vals = np.arange(len(k2), dtype=float) + 1.0
    lev2, dsh, sv = orbits_to_shells(k2, deg, vals)
    assert np.all(np.diff(lev2) > 0) and dsh.sum() == 64
    i011 = [i for i in range(len(k2)) if sorted(rep[i]) == [0, 1, 1]][0]
    i002 = [i for i in range(len(k2)) if sorted(rep[i]) == [0, 0, 2]][0]
    assert abs(k2[i011] - k2[i002]) < 1e-12
    s = int(np.argmin(np.abs(lev2 - k2[i011])))
    assert dsh[s] == deg[i011] + deg[i002]
    want = (vals[i011] * deg[i011] + vals[i002] * deg[i002]) / (deg[i011] + deg[i002])
    assert abs(sv[s] - want) <= 1e-15 * want
    # the degeneracy-weighted total is kept, and a stack of arrays maps row by row
    assert abs(np.dot(sv, dsh) - np.dot(vals, deg)) <= 1e-12 * np.dot(vals, deg)
    _, _, sv2 = orbits_to_shells(k2, deg, np.stack([vals, 2 * vals]))
    assert np.allclose(sv2[1], 2 * sv)
