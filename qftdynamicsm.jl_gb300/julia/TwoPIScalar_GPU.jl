###############################################################################################################################
# TwoPIScalar_GPU.jl -- GPU numerics for TwoPIScalar backed by libkb2pi (include/kb2pi.h)
#
# Drop-in Numerics for the reference's own simulation types: with this file included after
# TwoPIScalar_Modelfile.jl and parameters["Num"] = "GPU" (plain FP64) or "GPUmixed", the unchanged
# drivers (G_SimulationArgs.jl, TwoPIScalar_Testhelpers.jl, TwoPIScalar_Bechmark.jl) run
#   QFTdynamicsProblem -> QFTdynamicsSolution -> initialize! -> evolve!/measure!
# with every evolve! step on the GPU. The host keeps only what the reference computes on the host:
# parameters, occupation numbers, gap mass. Momentum shells are exact cubic orbits (kb_get_orbits);
# getindex on the simulation data pulls single elements from the device history.
#
# Not executed in this repository (no Julia toolchain on the build or GPU machines); the same C ABI
# is exercised from Python by the parity tests.
###############################################################################################################################
using Libdl

const libkb2pi = get(ENV, "KB2PI_LIB", joinpath(@__DIR__, "..", "kb2pi", "libkb2pi.so"))

struct KbParams
    Ns::Int32; sdim::Int32; M::Int32; N::Int32; pexp::Int32; precision::Int32; device::Int32; flags::Int32
    dt::Float64; lambda::Float64; mass2::Float64; mass::Float64
end

mutable struct KbMeasScalars
    time::Float64; E::Float64; E_pot::Float64; E_kin::Float64; E_mem::Float64; M2::Float64
end
KbMeasScalars() = KbMeasScalars(0, 0, 0, 0, 0, 0)

kbcheck(rc, h) = rc == 0 || error("libkb2pi: ", unsafe_string(ccall((:kb_last_error, libkb2pi), Cstring, (Ptr{Cvoid},), h)))

# Numerics selector next to TwoPIScalarCPUfull/CPUred (TwoPIScalar_Problemdefinition.jl:92-106)
struct TwoPIScalarGPU <: TwoPIScalarNumerics
    nchunks::Int       # kept for the parameter interface; the GPU ignores it
    precision::Int32   # 0 = FP64, 1 = mixed
end

# SimData: an opaque handle to the device-resident history, a subtype of the reference's
# abstract TwoPIScalarSimDataGPU (TwoPIScalar_SimDataStruct.jl:58)
mutable struct TwoPIScalarSimDataGPUkb <: TwoPIScalarSimDataGPU
    h::Ptr{Cvoid}
    S::Int
    kL2values::Vector{Float64}
    deg::Vector{Int64}
    orbit_of_site::Vector{Int32}
    NstepsinMemory::Int
    Nx::Int
    sdim::Int
    hartreemass2::Vector{Float64}
    function TwoPIScalarSimDataGPUkb(problem)
        d, m = problem.disc, problem.model
        pexp = problem.pexp isa TwoPIScalarLambdaLO ? 0 : problem.pexp isa TwoPIScalarLambdaNLOclassical ? 2 :
               problem.pexp isa TwoPIScalarNinverseLO ? 3 : problem.pexp isa TwoPIScalarNinverseNLO ? 4 : 1
        p = Ref(KbParams(d.Nx, d.sdim, problem.simsetup.NstepsinMemory, m.ONgroup, pexp, problem.num.precision, 0, 0,
                         d.dt, m.Lambda, m.Mass2, d.Mass))
        hr = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:kb_create, libkb2pi), Cint, (Ref{KbParams}, Ref{Ptr{Cvoid}}), p, hr)
        kbcheck(rc, C_NULL)
        S = Ref{Int32}(0)
        kbcheck(ccall((:kb_num_orbits, libkb2pi), Cint, (Ptr{Cvoid}, Int32, Ref{Int32}), hr[], 0, S), hr[])
        k2 = zeros(S[]); deg = zeros(Int64, S[]); rep = zeros(Int32, 3 * S[])
        kbcheck(ccall((:kb_get_orbits, libkb2pi), Cint, (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Float64}, Ptr{Int64}),
                      hr[], 0, rep, k2, deg), hr[])
        oos = zeros(Int32, d.Nx^d.sdim)
        kbcheck(ccall((:kb_site_orbits, libkb2pi), Cint, (Ptr{Cvoid}, Int32, Ptr{Int32}), hr[], 0, oos), hr[])
        sd = new(hr[], S[], k2, deg, oos, problem.simsetup.NstepsinMemory, d.Nx, d.sdim, [0.0])
        finalizer(x -> ccall((:kb_destroy, libkb2pi), Cvoid, (Ptr{Cvoid},), x.h), sd)
        return sd
    end
end

# SymMatrix-style getindex (DefSimDataElements.jl:185-208): F[i,j] as an orbit vector, F[i,j,site]
struct KbField; sd::TwoPIScalarSimDataGPUkb; which::Int32; end
Base.getproperty(sd::TwoPIScalarSimDataGPUkb, s::Symbol) =
    s === :F ? KbField(sd, 0) : s === :r ? KbField(sd, 1) : getfield(sd, s)
function Base.getindex(f::KbField, i::Int, j::Int)
    out = zeros(f.sd.S)
    kbcheck(ccall((:kb_get, libkb2pi), Cint, (Ptr{Cvoid}, Int32, Int32, Int32, Int32, Ptr{Float64}),
                  f.sd.h, 0, f.which, i, j, out), f.sd.h)
    return out   # rho values are the true antisymmetric rho(i,j); no thesign needed
end
Base.getindex(f::KbField, i::Int, j::Int, site::Int) = f[i, j][f.sd.orbit_of_site[site] + 1]

# getTwoPIScalarTmpData (TwoPIScalar_SimDataStruct.jl:710-721): the GPU keeps its scratch in the handle.
# getTwoPISimData (:669-708) branches on typeof(problem.num); its GPU branch is
#     if typeof(problem.num) == QFTdynamics.TwoPIScalarGPU simdata = TwoPIScalarSimDataGPUkb(problem) end
getTwoPIScalarTmpData(simdata::TwoPIScalarSimDataGPUkb, problem::QFTdynamicsProblem) = nothing

# initialize! (TwoPIScalar_Initialization.jl:289-325): occupation and gap mass on the host, rows on the GPU
function initialize!(thesolution::QFTdynamicsSolutionTwoPIScalar, tmpdata::Nothing)
    @unpack problem, simdata = thesolution
    @unpack model, pexp, disc, init, simsetup = problem
    if isnewsimulation(simsetup)
        if init isa TwoPIScalarGauss
            # initSimData! for TwoPIScalarGauss (TwoPIScalar_Initialization.jl:95-112): the same three
            # rows at every momentum, passed as rows (kb_init_rows)
            S = simdata.S
            F11 = fill(init.xi^2, S)
            F21 = init.xi * init.eta * disc.dt .+ F11
            F22 = (init.eta^2 + init.sig^2 / (4 * init.xi^2)) * disc.dt^2 .- F11 .+ 2 .* F21
            kbcheck(ccall((:kb_init_rows, libkb2pi), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                          simdata.h, 0, F11, F21, F22), simdata.h)
        else
            n = getparticlenr_orbits(init, disc, simdata.kL2values)
            initmass = (model isa Phi4Tachyonic || init isa TwoPIScalarQuench || init isa TwoPIScalarTopHatT1 ||
                        init isa TwoPIScalarThermal || init isa TwoPIScalarBox) ?
                       disc.Mass : getGapMass_orbits(model, pexp, disc, n, simdata)
            kbcheck(ccall((:kb_init, libkb2pi), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Float64),
                          simdata.h, 0, n, initmass), simdata.h)
        end
    end
    simsetup.lastEvolStep = 2
    measure!(thesolution, 2)
end

# evolve! (TwoPIScalar_Evolution.jl:924-981)
function evolve!(thesolution::QFTdynamicsSolutionTwoPIScalar, tmpdata::Nothing, t)
    kbcheck(ccall((:kb_step, libkb2pi), Cint, (Ptr{Cvoid}, Int32), thesolution.simdata.h, t), thesolution.simdata.h)
    thesolution.problem.simsetup.lastEvolStep = t
end

# createMeasurement (TwoPIScalar_Measurement.jl:31-99) from the device measurement
function createMeasurement(t::Int64, model::TwoPIScalarPhi4, simdata::TwoPIScalarSimDataGPUkb,
                           disc::TwoPIScalarDiscretization, pexp::TwoPIScalarPertExpansion)
    S = simdata.S
    s = Ref(KbMeasScalars())
    F = zeros(S); ddF = zeros(S); n = zeros(S); omega = zeros(S); c = zeros(S)
    kbcheck(ccall((:kb_measure, libkb2pi), Cint,
                  (Ptr{Cvoid}, Int32, Int32, Ref{KbMeasScalars}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                   Ptr{Float64}), simdata.h, 0, t, s, F, ddF, n, omega, c), simdata.h)
    meas = MeasurementTwoPIScalar{S, disc.NstepsinMemory}()
    meas.time, meas.E, meas.E_pot, meas.E_kin, meas.E_mem, meas.M2 = s[].time, s[].E, s[].E_pot, s[].E_kin, s[].E_mem, s[].M2
    meas.F, meas.ddF, meas.n, meas.omega, meas.c = F, ddF, n, omega, c
    meas.r = zeros(S)
    if t >= 3
        nw = t - max(1, t - simdata.NstepsinMemory + 1)
        meas.Fonet = zeros(nw); meas.ronet = zeros(nw); meas.SigF = zeros(nw); meas.Sigr = zeros(nw)
        kbcheck(ccall((:kb_get_traces, libkb2pi), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                      Ptr{Float64}), simdata.h, 0, meas.Fonet, meas.ronet, meas.SigF, meas.Sigr), simdata.h)
    end
    return meas
end

# Pipelined measurement for a driver loop that evolves step t+1 before it reads
# step t: call measure_enqueue(simdata, t) right after evolve!(..., t), and
# measure_take(simdata, t) (scalars and per-orbit arrays, as kb_measure) once
# step t+1 has been issued.
measure_enqueue(simdata::TwoPIScalarSimDataGPUkb, t) =
    kbcheck(ccall((:kb_measure_enqueue, libkb2pi), Cint, (Ptr{Cvoid}, Int32, Int32), simdata.h, 0, t), simdata.h)

function measure_take(simdata::TwoPIScalarSimDataGPUkb, t)
    S = simdata.S
    s = Ref(KbMeasScalars())
    F = zeros(S); ddF = zeros(S); n = zeros(S); omega = zeros(S); c = zeros(S)
    kbcheck(ccall((:kb_measure_take, libkb2pi), Cint,
                  (Ptr{Cvoid}, Int32, Int32, Ref{KbMeasScalars}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                   Ptr{Float64}), simdata.h, 0, t, s, F, ddF, n, omega, c), simdata.h)
    return s[], F, ddF, n, omega, c
end

# occupation per orbit, k2s = lev2 of every orbit (getparticlenr, TwoPIScalar_Initialization.jl:133-203)
getparticlenr_orbits(init::TwoPIScalarParticle, disc, k2s) = fill(Float64(init.n), length(k2s))
getparticlenr_orbits(init::TwoPIScalarThermal, disc, k2s) =
    [1 / (exp(sqrt(k2 + disc.Mass^2) / (init.T * disc.Mass)) - 1) for k2 in k2s]
getparticlenr_orbits(init::TwoPIScalarTsunami, disc, k2s) = [5 * exp(-(sqrt(k2) - 1)^2 / (2 * 0.2^2)) for k2 in k2s]
getparticlenr_orbits(init::TwoPIScalarQuench, disc, k2s) = zeros(length(k2s))
# TopHat states (:142-190): the reference fills eta between the lev2-sorted shells closest to
# lo * sdim * Mass^2 and hi * sdim * Mass^2; on orbits that is every orbit whose lev2 lies between
# those two shell values (the levels are the distinct lev2 values)
function tophat_orbits(disc, k2s, lo, hi, eta)
    levels = sort(unique(k2s))
    k2min = levels[argmin(abs.(levels .- lo * disc.sdim * disc.Mass^2))]
    k2max = levels[argmin(abs.(levels .- hi * disc.sdim * disc.Mass^2))]
    return [(k2min <= k2 <= k2max) ? Float64(eta) : 0.0 for k2 in k2s]
end
getparticlenr_orbits(init::TwoPIScalarTopHatT1, disc, k2s) = tophat_orbits(disc, k2s, 0.68, 2.04, 2)
getparticlenr_orbits(init::TwoPIScalarTopHatT2, disc, k2s) = tophat_orbits(disc, k2s, 0.0, 1.9, 1.85)
getparticlenr_orbits(init::TwoPIScalarTopHatT3, disc, k2s) = tophat_orbits(disc, k2s, 2.04, 2.72, 1.6)

# getGapMass (TwoPIScalar_Initialization.jl:250-266) summed over orbits with their degeneracy
function getGapMass_orbits(model, pexp, disc, n, simdata)
    g(x) = sum((1 / sqrt(k2 + x^2)) * (nn + 0.5) * dg for (k2, nn, dg) in zip(simdata.kL2values, n, simdata.deg)) *
           disc.ivol * Hartreeprefactor(model, pexp) + model.Mass2 - x^2
    D(f) = x -> ForwardDiff.derivative(f, float(x))
    return find_zero((g, D(g)), 0.5, Roots.Newton())
end

# Gradients by the discrete adjoint (kb_adjoint): L = sum_k w_n[k] n(k, t_final) + w_E E(t_final) on orbits,
# for the run started from occupation n_init at init_mass. A handle with NstepsinMemory M and extra ring
# slots (kb_params.flags) >= ckpt_every is created per call; its state is consumed.
function kb_loss_and_grad(problem, n_init::Vector{Float64}, init_mass, t_final, w_n, w_E; ckpt_every = 20)
    d, m = problem.disc, problem.model
    pexp = problem.pexp isa TwoPIScalarLambdaLO ? 0 : (problem.pexp isa TwoPIScalarLambdaNLOclassical ? 2 : 1)
    p = Ref(KbParams(d.Nx, d.sdim, problem.simsetup.NstepsinMemory, m.ONgroup, pexp, 0, 0, ckpt_every,
                     d.dt, m.Lambda, m.Mass2, d.Mass))
    hr = Ref{Ptr{Cvoid}}(C_NULL)
    kbcheck(ccall((:kb_create, libkb2pi), Cint, (Ref{KbParams}, Ref{Ptr{Cvoid}}), p, hr), C_NULL)
    gl = Ref(0.0); gm = Ref(0.0); gi = Ref(0.0); L = Ref(0.0); gn = zeros(length(n_init))
    try
        kbcheck(ccall((:kb_adjoint, libkb2pi), Cint,
                      (Ptr{Cvoid}, Ptr{Float64}, Float64, Int32, Ptr{Float64}, Float64, Int32,
                       Ref{Float64}, Ref{Float64}, Ptr{Float64}, Ref{Float64}, Ref{Float64}),
                      hr[], n_init, init_mass, t_final, w_n === nothing ? C_NULL : w_n, w_E, ckpt_every,
                      gl, gm, gn, gi, L), hr[])
    finally
        ccall((:kb_destroy, libkb2pi), Cvoid, (Ptr{Cvoid},), hr[])
    end
    return L[], (lambda = gl[], mass2 = gm[], n_init = gn, init_mass = gi[])
end

# ChainRulesCore rrule: late-time loss as a function of (lambda, m^2, n_init) with the adjoint as pullback.
# `kb_late_time_loss(problem, lambda, mass2, n_init, init_mass, t_final, w_n, w_E)` runs the forward pass.
# ChainRulesCore and ConstructionBase are already in the reference's Manifest.toml (as indirect
# dependencies, :136 and :210); add both to Project.toml [deps] with this file.
using ChainRulesCore
using ConstructionBase: setproperties
function kb_late_time_loss(problem, lambda, mass2, n_init, init_mass, t_final, w_n, w_E)
    pr = setproperties(problem, model = setproperties(problem.model, Lambda = lambda, Mass2 = mass2))
    return first(kb_loss_and_grad(pr, n_init, init_mass, t_final, w_n, w_E))
end
function ChainRulesCore.rrule(::typeof(kb_late_time_loss), problem, lambda, mass2, n_init, init_mass, t_final, w_n, w_E)
    pr = setproperties(problem, model = setproperties(problem.model, Lambda = lambda, Mass2 = mass2))
    L, g = kb_loss_and_grad(pr, n_init, init_mass, t_final, w_n, w_E)
    pullback(dL) = (NoTangent(), NoTangent(), dL * g.lambda, dL * g.mass2, dL .* g.n_init, dL * g.init_mass,
                    NoTangent(), NoTangent(), NoTangent())
    return L, pullback
end
