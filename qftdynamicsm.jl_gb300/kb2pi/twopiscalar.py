"""Host mirror of the reference's TwoPIScalar simulation interface over libkb2pi.

The reference drives a simulation as (G_SimulationArgs.jl:86-106)

    theproblem = QFTdynamicsProblem(modelfile, parameters)
    thesolution, tmpdata = QFTdynamicsSolution(modelfile, theproblem)
    initialize!(thesolution, tmpdata)
    for t in lastEvolStep+1 : Nsteps+2
        evolve!(thesolution, tmpdata, t)
        (t-2) % NstepsbetweenNmeas == 0 && measure!(thesolution, t)

This module keeps those names (``initialize``, ``evolve``, ``measure`` stand
for the Julia bang functions) and their argument meaning, with the numerics
selected by ``parameters["Num"]``: "GPU" (plain FP64) or "GPUmixed". The host
side computes only what the reference computes on the host: parameters,
renormalised mass, occupation numbers and the gap mass. Every time step runs
in libkb2pi on the GPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import capi

# ---------------------------------------------------------------------------
# problem definition (TwoPIScalar_Problemdefinition.jl, _Modelfile.jl)
# ---------------------------------------------------------------------------
PEXP = {"LambdaLO": capi.KB_PEXP_LO, "LambdaNLO": capi.KB_PEXP_NLO_QUANTUM,
        "LambdaNLOclassical": capi.KB_PEXP_NLO_CLASSICAL, "NinverseLO": capi.KB_PEXP_NINV_LO,
        "NinverseNLO": capi.KB_PEXP_NINV_NLO}
NUM = {"GPU": capi.KB_PREC_FP64, "GPUfull": capi.KB_PREC_FP64, "GPUmixed": capi.KB_PREC_MIXED}


class TwoPIScalarfile:
    """Model file selector (TwoPIScalar_Modelfile.jl:3-4)."""


@dataclass
class Phi4:
    Lambda: float
    ONgroup: int
    Mass2: float
    tachyonic: bool = False


@dataclass
class Discretization:
    Mass: float
    Nx: int
    sdim: int
    Nsteps: int
    dt: float
    vol: int
    ivol: float
    NstepsinMemory: int
    Nmeas: int


@dataclass
class SimSetup:
    Nsteps: int = 0
    Nmeas: int = 0
    NstepsbetweenNmeas: int = 0
    lastEvolStep: int = 0
    NstepsinMemory: int = 0


@dataclass
class Init:
    kind: str
    T: float = 0.0
    n: float = 0.0
    xi: float = 0.0
    eta: float = 0.0
    sig: float = 0.0


@dataclass
class QFTdynamicsProblem:
    model: Phi4
    pexp: str
    disc: Discretization
    init: Init
    reno: str
    num: str
    simsetup: SimSetup


def check_parameters(parameters: dict) -> None:
    """check_parameters! (src/DefAbstractSimSetup.jl:21-31)."""
    if parameters["NstepsinMemory"] == 0:
        parameters["NstepsinMemory"] = parameters["Nsteps"] + 2
    if parameters["Nmeas"] == 0:
        parameters["Nmeas"] = parameters["Nsteps"]


def lattice_orbits(Ns: int):
    """Cubic orbits of the Ns^3 lattice: (rep, lev2, deg), numbered as libkb2pi does."""
    H = Ns // 2 + 1
    reps, k2, deg = [], [], []
    mult = lambda x: 1 if (x == 0 or 2 * x == Ns) else 2  # noqa: E731
    for c in range(H):
        for b in range(c + 1):
            for a in range(b + 1):
                reps.append((a, b, c))
                k2.append(sum(4.0 * math.sin(math.pi * v / Ns) ** 2 for v in (a, b, c)))
                nperm = 1 if a == b == c else (3 if (a == b or b == c) else 6)
                deg.append(nperm * mult(a) * mult(b) * mult(c))
    return np.array(reps, np.int32), np.array(k2), np.array(deg, np.int64)


def hartree_prefactor(model: Phi4, pexp: str) -> float:
    """Hartreeprefactor (TwoPIScalar_Initialization.jl:245-247): lambda/6 for NinverseLO,
    lambda (N+2)/(6N) for the lambda expansion and NinverseNLO."""
    if pexp == "NinverseLO":
        return model.Lambda * (1 / 6)
    return model.Lambda * (model.ONgroup + 2) / (6 * model.ONgroup)


def getct(model: Phi4, pexp: str, disc: Discretization, k2, deg) -> float:
    """Mass counterterm (TwoPIScalar_ModelExpansionRenormalization.jl:38-47)."""
    ct = 0.0
    for kk, dg in zip(k2, deg):
        omega = math.sqrt(kk + disc.Mass ** 2)
        ct -= (0.5 / omega) * dg
    return ct * (hartree_prefactor(model, pexp) * disc.ivol)


def Renormalize(model: Phi4, pexp: str, reno: str, disc: Discretization, k2, deg) -> Phi4:
    """Renormalize (TwoPIScalar_ModelExpansionRenormalization.jl:18-36)."""
    if reno == "RNone":
        return model
    if reno == "RMass":
        ct = getct(model, pexp, disc, k2, deg)
        if model.tachyonic:
            return Phi4(model.Lambda, model.ONgroup, -model.Mass2 + ct, True)
        return Phi4(model.Lambda, model.ONgroup, model.Mass2 + ct, False)
    raise ValueError(f"unknown renormalisation {reno}")


def getparticlenr(init: Init, disc: Discretization, k2) -> np.ndarray:
    """getparticlenr per orbit (TwoPIScalar_Initialization.jl:133-203).

    The reference indexes momentum shells sorted by lev2 and selects the
    TopHat ranges by the shells closest to k2min/k2max; on orbits the same
    rule selects every orbit whose lev2 lies between those two shell values.
    Tsunami is declared but not implemented upstream
    (TwoPIScalar_Problemdefinition.jl:81); it is defined here as
    n(p) = 5 exp(-(|p| - 1)^2 / (2 * 0.2^2)) with |p| = sqrt(lev2), to which
    initSimData! adds the vacuum 1/2.
    """
    k2 = np.asarray(k2)
    if init.kind == "Pnr":
        return init.n * np.ones_like(k2)
    if init.kind == "Thermal":
        return 1.0 / (np.exp(np.sqrt(k2 + disc.Mass ** 2) / (init.T * disc.Mass)) - 1.0)
    if init.kind in ("TopHatT1", "TopHatT2", "TopHatT3"):
        lo, hi, eta = {"TopHatT1": (0.68, 2.04, 2.0), "TopHatT2": (0.0, 1.9, 1.85),
                       "TopHatT3": (2.04, 2.72, 1.6)}[init.kind]
        levels = np.unique(k2)
        k2min = levels[np.argmin(np.abs(levels - lo * disc.sdim * disc.Mass ** 2))]
        k2max = levels[np.argmin(np.abs(levels - hi * disc.sdim * disc.Mass ** 2))]
        return np.where((k2 >= k2min) & (k2 <= k2max), eta, 0.0)
    if init.kind == "Quench":
        return np.zeros_like(k2)
    if init.kind == "Tsunami":
        return 5.0 * np.exp(-((np.sqrt(k2) - 1.0) ** 2) / (2 * 0.2 ** 2))
    raise ValueError(f"no occupation profile for init {init.kind}")


def getGapMass(model: Phi4, pexp: str, disc: Discretization, n, k2, deg, x0: float = 0.5) -> float:
    """getGapMass (TwoPIScalar_Initialization.jl:250-266): Newton from x0 = 0.5."""
    n = np.asarray(n)
    pref = hartree_prefactor(model, pexp)
    w = (n + 0.5) * np.asarray(deg, np.float64)

    def g(x):
        om2 = np.asarray(k2) + x * x
        res = np.sum((1.0 / np.sqrt(om2)) * w) * disc.ivol * pref + model.Mass2 - x * x
        d = np.sum(-x / (om2 * np.sqrt(om2)) * w) * disc.ivol * pref - 2 * x
        return res, d

    x = x0
    for _ in range(200):
        f, d = g(x)
        if f == 0.0:
            break
        xn = x - f / d
        if abs(xn - x) <= 4 * np.finfo(float).eps * abs(xn):
            x = xn
            break
        x = xn
    return x


def make_problem(modelfile: TwoPIScalarfile, parameters: dict) -> QFTdynamicsProblem:
    """QFTdynamicsProblem(modelfile, parameters) (TwoPIScalar_Modelfile.jl:46-124)."""
    check_parameters(parameters)
    Nx, sdim = parameters["Nx"], parameters["sdim"]
    disc = Discretization(parameters["Mass"], Nx, sdim, parameters["Nsteps"], parameters["dt"], Nx ** sdim,
                          1 / (Nx ** sdim), parameters["NstepsinMemory"], parameters["Nmeas"])
    mod = parameters.get("Mod", "phi4")
    model = Phi4(parameters["Lambda"], parameters["ONgroup"], parameters["Mass"] ** 2, mod == "phi4tachyonic")
    init = Init(parameters["init"], T=parameters.get("T", 0.0), n=parameters.get("n", 0.0),
                xi=parameters.get("xi", 0.0), eta=parameters.get("eta", 0.0), sig=parameters.get("sig", 0.0))
    pexp = parameters["Pexp"]
    if pexp not in PEXP:
        raise ValueError(f"Pexp {pexp} is not provided by the GPU numerics")
    num = parameters.get("Num", "GPU")
    if num not in NUM:
        raise ValueError(f"Num {num}: the GPU numerics are 'GPU' (FP64) and 'GPUmixed'")
    ss = SimSetup()
    ss.NstepsinMemory = parameters["NstepsinMemory"]
    ss.NstepsbetweenNmeas = int(parameters["Nsteps"] // parameters["Nmeas"])
    ss.Nsteps = ss.NstepsbetweenNmeas * parameters["Nmeas"]
    ss.Nmeas = parameters["Nmeas"]
    _, k2, deg = lattice_orbits(Nx)
    renomodel = Renormalize(model, pexp, parameters["Reno"], disc, k2, deg)
    return QFTdynamicsProblem(renomodel, pexp, disc, init, parameters["Reno"], num, ss)


# Julia overloads QFTdynamicsProblem on the model file; keep that spelling too.
def QFTdynamicsProblem_(modelfile, parameters):  # pragma: no cover - alias
    return make_problem(modelfile, parameters)


@dataclass
class QFTdynamicsSolutionTwoPIScalar:
    problem: QFTdynamicsProblem
    simdata: "GPUSimData"
    measurearray: list = field(default_factory=list)


class GPUSimData:
    """TwoPIScalarSimData backed by a libkb2pi handle (device-resident history)."""

    def __init__(self, problem: QFTdynamicsProblem, device: int = 0):
        d = problem.disc
        p = capi.KbParams(Ns=d.Nx, sdim=d.sdim, M=d.NstepsinMemory, N=problem.model.ONgroup,
                          pexp=PEXP[problem.pexp], precision=NUM[problem.num], device=device, flags=0,
                          dt=d.dt, lam=problem.model.Lambda, mass2=problem.model.Mass2, mass=d.Mass)
        self.handle = capi.Handle([p])
        self.rep, self.kL2values, self.deg = self.handle.orbits(0)
        self.NstepsinMemory = d.NstepsinMemory
        self.Nx, self.sdim = d.Nx, d.sdim

    @property
    def indices(self):
        return list(self.handle.window(0))

    def F(self, a, b):
        """simdata.F[a,b] on orbits (SymMatrix getindex, DefSimDataElements.jl:185-195)."""
        return self.handle.get(0, 0, a, b)

    def r(self, a, b):
        """True rho(a,b) (r[a,b] * thesign(a,b) in the reference)."""
        return self.handle.get(0, 1, a, b)


def QFTdynamicsSolution(modelfile: TwoPIScalarfile, problem: QFTdynamicsProblem, device: int = 0):
    """QFTdynamicsSolution (TwoPIScalar_Modelfile.jl:133-143): returns (solution, tmpdata)."""
    simdata = GPUSimData(problem, device)
    sol = QFTdynamicsSolutionTwoPIScalar(problem, simdata, [None] * (problem.simsetup.Nmeas + 1))
    return sol, None  # the GPU backend keeps its scratch inside the handle


def initialize(thesolution: QFTdynamicsSolutionTwoPIScalar, tmpdata=None) -> None:
    """initialize! (TwoPIScalar_Initialization.jl:289-325)."""
    pr = thesolution.problem
    sd = thesolution.simdata
    model, disc, init = pr.model, pr.disc, pr.init
    if pr.simsetup.lastEvolStep == 0:
        if init.kind == "Gauss":
            # initSimData! for TwoPIScalarGauss (TwoPIScalar_Initialization.jl:95-112)
            S = len(sd.kL2values)
            F11 = np.full(S, init.xi ** 2)
            F21 = init.xi * init.eta * disc.dt + F11
            F22 = (init.eta ** 2 + init.sig ** 2 / (4 * init.xi ** 2)) * disc.dt ** 2 - F11 + 2 * F21
            sd.handle.init_rows(0, F11, F21, F22)
        else:
            n = getparticlenr(init, disc, sd.kL2values)
            if model.tachyonic or init.kind in ("Quench", "TopHatT1", "Thermal", "Box"):
                initmass = disc.Mass
            else:  # Tsunami and the generic branch use the gap mass (:309-319)
                initmass = getGapMass(model, pr.pexp, disc, n, sd.kL2values, sd.deg)
            sd.handle.init(0, n, initmass)
    pr.simsetup.lastEvolStep = 2
    measure(thesolution, 2)


def evolve(thesolution: QFTdynamicsSolutionTwoPIScalar, tmpdata, t: int) -> None:
    """evolve! (TwoPIScalar_Evolution.jl:924-981) on the GPU."""
    thesolution.simdata.handle.step(t)
    thesolution.problem.simsetup.lastEvolStep = t


def createMeasurement(t: int, thesolution: QFTdynamicsSolutionTwoPIScalar) -> dict:
    """createMeasurement (TwoPIScalar_Measurement.jl:31-99): scalars, per-orbit arrays, traces."""
    h = thesolution.simdata.handle
    m = h.measure(0, t)
    m["r"] = np.zeros_like(m["F"])  # rho(t-1,t-1) = 0
    if t >= 3:
        m.update(h.traces(0))
    return m


def measure(thesolution: QFTdynamicsSolutionTwoPIScalar, t: int) -> None:
    """measure! (TwoPIScalar_Measurement.jl:223-228)."""
    ss = thesolution.problem.simsetup
    thesolution.measurearray[int((t - 2) / ss.NstepsbetweenNmeas)] = createMeasurement(t, thesolution)


def evolve_recorded(thesolution: QFTdynamicsSolutionTwoPIScalar, tlast: int) -> None:
    """evolve! from lastEvolStep + 1 to tlast with measure! of every NstepsbetweenNmeas-th
    step taken from the device measurement stream (kb_steps_recorded): one graph launch per
    step and a single host read at the end. The records carry the scalars and per-orbit
    arrays of createMeasurement; the site-1 traces are only available for the last step."""
    ss = thesolution.problem.simsetup
    h = thesolution.simdata.handle
    t0 = ss.lastEvolStep + 1
    if tlast < t0:
        return
    for row in h.steps_recorded(t0, tlast - t0 + 1, ss.NstepsbetweenNmeas):
        m = row[0]
        t = m.pop("t")
        m["r"] = np.zeros_like(m["F"])
        thesolution.measurearray[int((t - 2) / ss.NstepsbetweenNmeas)] = m
    ss.lastEvolStep = tlast
    if (tlast - 2) % ss.NstepsbetweenNmeas == 0:
        thesolution.measurearray[int((tlast - 2) / ss.NstepsbetweenNmeas)].update(h.traces(0))


def run_simulation(parameters: dict, evolveto: int | None = None, device: int = 0, stream: bool = False):
    """TwoPIScalar_testevolution (TwoPIScalar_Testhelpers.jl:27-48) on the GPU numerics.
    stream=True takes the measurements from the device measurement stream."""
    problem = make_problem(TwoPIScalarfile(), parameters)
    sol, tmp = QFTdynamicsSolution(TwoPIScalarfile(), problem, device)
    initialize(sol, tmp)
    last = evolveto if evolveto is not None else problem.simsetup.Nsteps + 2
    if stream:
        evolve_recorded(sol, last)
        return sol
    for t in range(problem.simsetup.lastEvolStep + 1, last + 1):
        evolve(sol, tmp, t)
        if (t - 2) % problem.simsetup.NstepsbetweenNmeas == 0:
            measure(sol, t)
    return sol


# Measurearray serialisation. The reference saves Vector{MeasurementTwoPIScalar}
# with JLD (G_SimulationArgs.jl); here each record keeps its MeasurementTwoPIScalar
# field names (TwoPIScalar_Measurement.jl:2-23) in one .npz archive, with the
# simulation parameters as JSON, so analysis code can read GPU runs field by field.
MEASUREMENT_FIELDS = ("time", "E", "E_pot", "E_kin", "E_mem", "M2", "F", "ddF", "n", "omega", "c", "r",
                      "Fonet", "ronet", "SigF", "Sigr")


def save_measurearray(path: str, thesolution: QFTdynamicsSolutionTwoPIScalar, parameters: dict | None = None):
    import json

    arrays = {"parameters": np.array(json.dumps(parameters or {}))}
    count = 0
    for i, m in enumerate(thesolution.measurearray):
        if m is None:
            continue
        count += 1
        for k in MEASUREMENT_FIELDS:
            if k in m:
                arrays[f"{i}/{k}"] = np.asarray(m[k])
    arrays["indices"] = np.array([i for i, m in enumerate(thesolution.measurearray) if m is not None], dtype=np.int64)
    np.savez(path, **arrays)
    return count


def load_measurearray(path: str):
    """Returns (measurearray, parameters): a list with None where nothing was measured."""
    import json

    z = np.load(path, allow_pickle=False)
    idx = [int(i) for i in z["indices"]]
    out = [None] * ((max(idx) + 1) if idx else 0)
    for i in idx:
        rec = {}
        for k in MEASUREMENT_FIELDS:
            key = f"{i}/{k}"
            if key in z.files:
                v = z[key]
                rec[k] = float(v) if v.ndim == 0 else v
        out[i] = rec
    return out, json.loads(str(z["parameters"]))


def orbits_to_shells(k2, deg, values, rtol: float = 1e-12):
    """Per-orbit measurement arrays on FFTWhelper-style shells (one entry per distinct
    lev2, as the reference's MeasurementTwoPIScalar arrays index by `lev2`,
    TwoPIScalar_Measurement.jl:24-25, 31-33).

    Orbits whose lev2 agree to rtol form one shell; a shell's value is the
    degeneracy-weighted mean of its orbits' values, which is the mean over the
    shell's lattice sites (the CPUfull measurement averaged over the shell).
    Returns (lev2 per shell ascending, deg per shell, values per shell); `values`
    may be one array (S,) or a stack (..., S). FFTWhelper's own grouping rule is
    not vendored in the reference; grouping by equal lev2 is what its `lev2`
    field names."""
    k2 = np.asarray(k2, np.float64)
    deg = np.asarray(deg, np.float64)
    vals = np.asarray(values, np.float64)
    order = np.argsort(k2, kind="stable")
    ks = k2[order]
    new = np.ones(len(ks), bool)
    new[1:] = np.abs(np.diff(ks)) > rtol * np.maximum(np.abs(ks[1:]), 1.0)
    shell_of_sorted = np.cumsum(new) - 1
    nshell = int(shell_of_sorted[-1]) + 1 if len(ks) else 0
    shell = np.empty(len(k2), np.int64)
    shell[order] = shell_of_sorted
    dsh = np.bincount(shell, weights=deg, minlength=nshell)
    lev2 = np.bincount(shell, weights=k2 * deg, minlength=nshell) / dsh
    flat = vals.reshape(-1, vals.shape[-1])
    out = np.stack([np.bincount(shell, weights=row * deg, minlength=nshell) / dsh for row in flat])
    return lev2, dsh.astype(np.int64), out.reshape(vals.shape[:-1] + (nshell,))
