"""
    NQCDGPU

GB300 ensemble algorithm for NQCDynamics.jl.

`EnsembleGB300` is a `SciMLBase.EnsembleAlgorithm`.  `run_dynamics`
(src/Ensembles/run_dynamics.jl:42-136) forwards its `ensemble_algorithm`
keyword to `SciMLBase.solve(ensemble_problem, algorithm, ensemble_algorithm;
trajectories, kwargs...)` (:91-97); with `ensemble_algorithm =
EnsembleGB300()` that call lands in the `SciMLBase.__solve` method below,
which runs the whole ensemble in the GB300 engine through `ccall` into
`libnqcd_gb300.so` (C ABI: include/nqcd_gpu.h) and returns the
`EnsembleSolution` whose `.u` `run_dynamics` reads (:131-135).

    using NQCDynamics, NQCDGPU
    sim = Simulation{FSSH}(Atoms(2000), TullyModelOne())
    res = run_dynamics(sim, (0.0, 3000.0), distribution; dt=1.0, trajectories=10_000,
                       output=OutputStateResolvedScattering1D(sim, :adiabatic),
                       reduction=MeanReduction(), ensemble_algorithm=EnsembleGB300(:fp32))

There is no CPU fallback: input the engine does not support raises an
`ArgumentError` before any `ccall`, and a missing library or GPU raises.

`KeyedStream` is the engine's random stream (Philox4x32-10 keyed by seed,
trajectory, step and stream) in Julia, and `install_keyed_hop_stream!`
makes the reference's own CPU integration draw its hop-test uniforms from it,
so that the reference and the plain FP64 GPU path consume the same numbers
and their hop sequences can be compared trajectory by trajectory.

The library is found through the environment variable `NQCD_GB300_LIB`
(default `libnqcd_gb300`, searched on the loader path).
"""
module NQCDGPU

using Random: Random
using Libdl: Libdl
using SciMLBase: SciMLBase
using Dictionaries: Dictionary
using NQCDynamics: NQCDynamics

export EnsembleGB300, install_keyed_hop_stream!, with_keyed_hops, keyed_fermi_dirac_state, keyed_noise_grid

# ---------------------------------------------------------------------------
# C ABI (include/nqcd_gpu.h)
# ---------------------------------------------------------------------------

const ABI_VERSION = Int32(111)

const METHOD_FSSH = Int32(1)
const METHOD_RPSH = Int32(2)
const METHOD_IESH = Int32(3)
const METHOD_MDEF = Int32(4)
const METHOD_EHRENFEST = Int32(5)
const METHOD_EHRENFEST_NA = Int32(6)

const MODEL_TULLY1 = Int32(1)
const MODEL_TULLY2 = Int32(2)
const MODEL_TULLY3 = Int32(3)
const MODEL_SPINBOSON = Int32(10)
const MODEL_NEWNS_ANDERSON = Int32(20)
const MODEL_NEWNS_ANDERSON_3D = Int32(21)

const PREC_FP64 = Int32(0)
const PREC_FP32 = Int32(1)
const PREC_FP32_KAHAN = Int32(2)

const INIT_GIVEN = Int32(0)
const INIT_ADIABATIC_PURE = Int32(1)
const INIT_DIABATIC_PURE = Int32(2)
const INIT_FERMI_DIRAC = Int32(3)

const SAMPLE_FIXED = Int32(0)
const SAMPLE_NORMAL = Int32(1)
const SAMPLE_UNIFORM = Int32(2)

# nqcd_config: same fields, order and types as the C struct (isbits, so Julia
# lays it out as C does).
struct NqcdConfig
    method::Int32
    model::Int32
    precision::Int32
    rescaling::Int32
    ndofs::Int32
    natoms::Int32
    nstates::Int32
    nbeads_max::Int32
    nparams::Int32
    params::Ptr{Float64}
    nbath::Int32
    bath_a::Ptr{Float64}
    bath_b::Ptr{Float64}
    masses::Ptr{Float64}
    beta::Float64
    ntraj_max::Int64
    init_kind::Int32
    init_state::Int32
    save_stride::Int32
    max_hops::Int32
    terminate_x::Float64
    gap_fp64::Float64
    traj_offset::Int64
    use_friction_surrogate::Int32
    exact_friction_every::Int32
    nelectrons::Int32
    exact_hop_probability::Int32
    reserved::NTuple{2,Int32}
    decoherence_C::Float64
    surrogate_tolerance::Float64
end

struct NqcdOutputs
    scattering::Ptr{Float64}
    population_correlation::Ptr{Float64}
    observables::Ptr{Float64}
    nsave::Int32
    reserved::Int32
end

struct NqcdStats
    traj_steps::Int64
    hops::Int64
    frustrated::Int64
    flagged::Int64
    device_ms::Float64
    kernel_ms::Float64
    wall_ms::Float64
    h2d_bytes::Int64
    d2h_bytes::Int64
    kernel_launches::Int32
    reserved::Int32
    exact_friction_evals::Int64
    surrogate_friction_evals::Int64
    unconverged_roots::Int64
    hop_evaluations::Int64
    propagator_terms::Int64
    electronics_fp64_steps::Int64
    surrogate_judged::Int64
    surrogate_rejected::Int64
    surrogate_max_rel_error::Float64
    surrogate_mean_rel_error::Float64
    overlap_factorizations::Int64
end

struct NqcdSampler
    kind::Int32
    reserved::Int32
    a::Float64
    b::Float64
end

struct NqcdMapping
    sb_lanes::Int32
    sb_block::Int32
    rp_lanes::NTuple{4,Int32}
    iesh_cores::Int32
    rp_one_launch::Int32
    iesh_lu_always::Int32
end

zero_stats() = NqcdStats(0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0.0, 0.0, 0)

"""
    config(; method, model, ndofs, natoms, nstates, ..., keep)

An `NqcdConfig` with the engine's defaults for every field not given.  The
arrays behind `params`, `bath_a`, `bath_b` and `masses` are pushed onto
`keep`, which the caller holds (`GC.@preserve`) while the handle is created.
"""
function config(; method, model, ndofs, natoms, nstates, params, masses, keep, precision=PREC_FP64,
                rescaling=Int32(0), nbeads_max=0, bath_a=Float64[], bath_b=Float64[], beta=0.0, ntraj_max,
                init_kind=INIT_ADIABATIC_PURE, init_state=0, save_stride=0, max_hops=0, terminate_x=0.0,
                gap_fp64=1e-3, traj_offset=0, use_friction_surrogate=0, exact_friction_every=0, nelectrons=0,
                exact_hop_probability=0, decoherence_C=0.0, surrogate_tolerance=0.0)
    p = collect(Float64, params)
    m = collect(Float64, masses)
    a = collect(Float64, bath_a)
    b = collect(Float64, bath_b)
    push!(keep, p, m, a, b)
    ptr(x) = isempty(x) ? Ptr{Float64}(C_NULL) : pointer(x)
    return NqcdConfig(method, model, precision, rescaling, ndofs, natoms, nstates, nbeads_max, length(p), ptr(p),
                      length(a), ptr(a), ptr(b), ptr(m), beta, ntraj_max, init_kind, init_state, save_stride,
                      max_hops, terminate_x, gap_fp64, traj_offset, use_friction_surrogate, exact_friction_every,
                      nelectrons, exact_hop_probability, (Int32(0), Int32(0)), decoherence_C,
                      surrogate_tolerance)
end

const LIBHANDLE = Ref{Ptr{Cvoid}}(C_NULL)

function library()
    if LIBHANDLE[] == C_NULL
        LIBHANDLE[] = Libdl.dlopen(get(ENV, "NQCD_GB300_LIB", "libnqcd_gb300"))
        v = ccall(Libdl.dlsym(LIBHANDLE[], :nqcd_version), Cint, ())
        v == ABI_VERSION || error("libnqcd_gb300 has ABI $v, this module binds $ABI_VERSION")
    end
    return LIBHANDLE[]
end

sym(name::Symbol) = Libdl.dlsym(library(), name)

struct EngineError <: Exception
    code::Int
    message::String
end
Base.showerror(io::IO, e::EngineError) = print(io, "nqcd engine error ", e.code, ": ", e.message)

last_error(h::Ptr{Cvoid}) = unsafe_string(ccall(sym(:nqcd_last_error), Cstring, (Ptr{Cvoid},), h))
check(h::Ptr{Cvoid}, rc::Integer) = rc == 0 ? nothing : throw(EngineError(rc, last_error(h)))

function create(cfg::NqcdConfig)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(C_NULL, ccall(sym(:nqcd_create), Cint, (Ref{NqcdConfig}, Ref{Ptr{Cvoid}}), cfg, h))
    return h[]
end

destroy(h::Ptr{Cvoid}) = ccall(sym(:nqcd_destroy), Cvoid, (Ptr{Cvoid},), h)

# ---------------------------------------------------------------------------
# KeyedStream: the engine's random stream (csrc/nqcd_math.h)
# ---------------------------------------------------------------------------

"""
    KeyedStream

Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC'11) keyed exactly as the
engine keys it: counter = (trajectory low word, trajectory high word, step,
stream), key = (seed low word, seed high word).  One block per (trajectory,
step, stream); streams: HOP 1 (hop test), INIT_STATE 2, NOISE 3 + 16 dof
(MDEF Wiener increments), INIT_FD 4 and 4 + 16 (Fermi-Dirac Metropolis),
INIT_POSITION 5, INIT_VELOCITY 6.
"""
module KeyedStream

const PHILOX_M0 = 0xD2511F53
const PHILOX_M1 = 0xCD9E8D57
const PHILOX_W0 = 0x9E3779B9
const PHILOX_W1 = 0xBB67AE85

const RNG_HOP = UInt32(1)
const RNG_INIT_STATE = UInt32(2)
const RNG_NOISE = UInt32(3)
const RNG_INIT_FD = UInt32(4)
const RNG_INIT_POSITION = UInt32(5)
const RNG_INIT_VELOCITY = UInt32(6)

# Known answers of Philox4x32-10 (Random123 test vectors): counter, key, output.
const KNOWN_ANSWERS = (
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF),
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
)

@inline function mulhilo(a::UInt32, b::UInt32)
    p = UInt64(a) * UInt64(b)
    return (p >> 32) % UInt32, p % UInt32
end

"""Ten rounds of Philox4x32 on counter (c0, c1, c2, c3) with key (k0, k1)."""
@inline function philox4x32_10(c0::UInt32, c1::UInt32, c2::UInt32, c3::UInt32, k0::UInt32, k1::UInt32)
    for _ in 1:10
        hi0, lo0 = mulhilo(PHILOX_M0, c0)
        hi1, lo1 = mulhilo(PHILOX_M1, c2)
        c0, c1, c2, c3 = hi1 ⊻ c1 ⊻ k0, lo1, hi0 ⊻ c3 ⊻ k1, lo0
        k0 += PHILOX_W0
        k1 += PHILOX_W1
    end
    return (c0, c1, c2, c3)
end

"""The block of (seed, trajectory, step, stream); trajectory is the global 0-based index."""
@inline block(seed::UInt64, traj::UInt64, step::UInt32, stream::UInt32) =
    philox4x32_10(traj % UInt32, (traj >> 32) % UInt32, step, stream, seed % UInt32, (seed >> 32) % UInt32)

"""53-bit uniform in [0, 1) from two words: the top 53 bits of (hi, lo) times 2^-53."""
@inline u53(hi::UInt32, lo::UInt32) = Float64(((UInt64(hi) << 32) | UInt64(lo)) >> 11) * 0x1p-53

"""The plain path's uniform (hop test, initial state, Metropolis)."""
@inline function uniform(seed, traj, step, stream)
    w = block(UInt64(seed), UInt64(traj), UInt32(step), UInt32(stream))
    return u53(w[1], w[2])
end

"""The FP32 paths' 24-bit uniform from the same block."""
@inline function uniform24(seed, traj, step, stream)
    w = block(UInt64(seed), UInt64(traj), UInt32(step), UInt32(stream))
    return Float32(w[1] >> 8) * Float32(0x1p-24)
end

"""
Standard normal of MDEF step `step` (1-based) and degree of freedom `dof`
(0-based): Box-Muller on one block, u1 = 1 - u53(w1, w2) in (0, 1],
u2 = u53(w3, w4).  Equal to the engine's draw to the rounding of log and cos.
"""
@inline function normal(seed, traj, step, dof)
    w = block(UInt64(seed), UInt64(traj), UInt32(step), RNG_NOISE + UInt32(16) * UInt32(dof))
    u1 = 1.0 - u53(w[1], w[2])
    u2 = u53(w[3], w[4])
    return sqrt(-2.0 * log(u1)) * cos(2.0 * pi * u2)
end

"""True when this implementation reproduces every known answer."""
function selftest()
    for (c, k, out) in KNOWN_ANSWERS
        philox4x32_10(c..., k...) == out || return false
    end
    return true
end

end # module KeyedStream

# ---------------------------------------------------------------------------
# The reference's hop draws from the keyed stream
# ---------------------------------------------------------------------------

const HOP_KEY = :nqcd_gb300_hop_key

mutable struct HopKey
    seed::UInt64
    traj::UInt64
    step::UInt32
end

"""
    with_keyed_hops(selection, seed; traj_offset=0)

Wrap the `prob_func` of an ensemble problem (the `Selection` that
`run_dynamics` builds, src/Ensembles/selections.jl) so that trajectory `i`
starts a hop key (seed, traj_offset + i - 1, step 0) in task-local storage.
SciMLBase runs a trajectory's `prob_func` and its `solve` in the same task
for `EnsembleSerial` and `EnsembleThreads`, so the key follows the
trajectory.
"""
struct KeyedSelection{S}
    selection::S
    seed::UInt64
    traj_offset::Int
end
with_keyed_hops(selection, seed; traj_offset=0) = KeyedSelection(selection, UInt64(seed), traj_offset)

function (k::KeyedSelection)(prob, i, repeat)
    task_local_storage(HOP_KEY, HopKey(k.seed, UInt64(k.traj_offset + i - 1), UInt32(0)))
    return k.selection(prob, i, repeat)
end

"""
The uniform for the current trajectory's next hop test.  The reference
tests for a hop once per step, so the n-th call of a trajectory is step n,
the same key the engine uses (its step counter is incremented before the
hop test).
"""
function next_hop_uniform()
    k = task_local_storage(HOP_KEY)::HopKey
    k.step += UInt32(1)
    return KeyedStream.uniform(k.seed, k.traj, k.step, KeyedStream.RNG_HOP)
end

"""
    install_keyed_hop_stream!()

Redefine the two places where the reference draws its hop-test uniform from
Julia's task-local RNG so that they draw `next_hop_uniform()` instead:

  * FSSH `select_new_state(sim, u)` (src/DynamicsMethods/SurfaceHoppingMethods/fssh.jl:110-121,
    the draw at :112): the first state m != s whose cumulative probability
    exceeds the draw;
  * IESH `iesh_check_hop!(u, t, integrator)` (iesh.jl:390-398, the draw at
    :393): the draw passed to the probability evaluation (its estimate screen)
    and to the cumulative selection over (electron, unoccupied state) pairs.

Everything else is unchanged.  Run the reference with the problem's
`prob_func` wrapped by `with_keyed_hops` (or call `keyed_run_dynamics`);
the plain FP64 GPU path with the same seed then sees the same uniforms, so
the two hop sequences can be compared trajectory by trajectory.  Initial
IESH occupations drawn by the reference's Metropolis sampler come from
Julia's RNG; `keyed_fermi_dirac_state` draws them from the keyed stream.
"""
function install_keyed_hop_stream!()
    SHM = NQCDynamics.DynamicsMethods.SurfaceHoppingMethods
    draw = next_hop_uniform
    @eval SHM begin
        function select_new_state(sim::NQCDynamics.AbstractSimulation{<:FSSH}, u)
            u_hop = $draw()
            s = sim.method.state
            for (m, cumulative) in enumerate(sim.method.hopping_probability)
                m == s && continue
                cumulative > u_hop && return m
            end
            return s
        end
        function iesh_check_hop!(u, t, integrator)::Bool
            sim = integrator.p
            ishoppingdisabled(sim.method) && return false
            u_hop = $draw()
            evaluate_hopping_probability!(sim, u, OrdinaryDiffEq.get_proposed_dt(integrator), u_hop)
            set_new_state!(sim.method, select_new_state(sim, u, u_hop))
            return sim.method.new_state != sim.method.state
        end
    end
    return nothing
end

"""
    keyed_run_dynamics(sim, tspan, distribution; seed, kwargs...)

`run_dynamics` with the hop draws keyed by (seed, trajectory, step): installs
the keyed hop stream and wraps the ensemble problem's selection.  Compare its
`OutputSurfaceHops` with the engine's hop log (`nqcd_get_hop_log`) of a plain
FP64 run with the same seed.
"""
function keyed_run_dynamics(sim, tspan, distribution; seed, trajectories=1, output=NQCDynamics.OutputFinal, kwargs...)
    install_keyed_hop_stream!()
    # run_dynamics has no hook for its prob_func, so the ensemble is assembled
    # from the reference's own pieces (run_dynamics.jl:74-89) with the
    # selection wrapped.
    selection = NQCDynamics.Ensembles.Selection(distribution, nothing, trajectories)
    u0 = NQCDynamics.Ensembles.sample_distribution(sim, distribution)
    problem = NQCDynamics.DynamicsMethods.create_problem(u0, float.(tspan), sim)
    outputs = output isa Tuple ? output : (output,)
    ens = SciMLBase.EnsembleProblem(problem; prob_func=with_keyed_hops(selection, seed),
                                    output_func=NQCDynamics.Ensembles.EnsembleSaver(outputs, true),
                                    reduction=NQCDynamics.Ensembles.SortByTrajectoryReduction())
    return SciMLBase.solve(ens, NQCDynamics.DynamicsMethods.select_algorithm(sim), SciMLBase.EnsembleSerial();
                           trajectories, kwargs...).u
end

"""
    keyed_fermi_dirac_state(energies, nelectrons, beta, seed, traj)

The engine's Fermi-Dirac Metropolis sampling of initial occupations
(the reference's src/DynamicsUtils/DynamicsUtils.jl:194-208 with keyed
draws): start from the lowest `nelectrons` states; for iteration it =
0 .. nstates * nelectrons - 1, block A = (seed, traj, it, 4) and B = (seed,
traj, it, 20); the electron is floor(u53(A1, A2) ne), the unoccupied state
(ascending order) floor(u53(A3, A4) n_unocc), accepted when
exp(-beta (E_j - E_i)) > u53(B1, B2).  Returns the sorted 1-based states.
"""
function keyed_fermi_dirac_state(energies::AbstractVector, nelectrons::Integer, beta::Real, seed, traj)
    N = length(energies)
    state = collect(1:nelectrons)
    for it in 0:(N * nelectrons - 1)
        a = KeyedStream.block(UInt64(seed), UInt64(traj), UInt32(it), KeyedStream.RNG_INIT_FD)
        b = KeyedStream.block(UInt64(seed), UInt64(traj), UInt32(it), KeyedStream.RNG_INIT_FD + UInt32(16))
        ua, ub, uc = KeyedStream.u53(a[1], a[2]), KeyedStream.u53(a[3], a[4]), KeyedStream.u53(b[1], b[2])
        ci = min(floor(Int, ua * nelectrons), nelectrons - 1) + 1
        unocc = setdiff(1:N, state)
        j = unocc[min(floor(Int, ub * length(unocc)), length(unocc) - 1) + 1]
        i = state[ci]
        if exp(-beta * (energies[j] - energies[i])) > uc
            state[ci] = j
        end
    end
    return sort!(state)
end

"""
    keyed_noise_grid(seed, traj, dt, nsteps, ndof)

Times and Wiener values W(t_k) = sqrt(dt) sum_{n <= k} xi_n with xi_n the
engine's keyed normals of step n, one per degree of freedom, for a
`NoiseGrid(t, W)` passed to the MDEF integrator as `noise`.  The increment of
step n divided by sqrt(dt) is then the engine's draw to rounding.
"""
function keyed_noise_grid(seed, traj, dt::Real, nsteps::Integer, ndof::Integer)
    W = [zeros(ndof)]
    for n in 1:nsteps
        xi = [KeyedStream.normal(seed, traj, n, d) for d in 0:(ndof - 1)]
        push!(W, W[end] .+ sqrt(dt) .* xi)
    end
    return collect(0:nsteps) .* dt, W
end

# ---------------------------------------------------------------------------
# EnsembleGB300
# ---------------------------------------------------------------------------

"""
    EnsembleGB300(precision=:fp32; seed=rand(UInt64), max_hops=0, gap_fp64=1e-3)

Run a whole ensemble in the GB300 engine.  `precision`: `:fp64` (the plain
path, FP64 throughout, the reference's operation order), `:fp32` or
`:fp32_kahan` (the fast paths; every fast result has a stated error against
`:fp64`).  `seed` keys the engine's random stream.
"""
struct EnsembleGB300 <: SciMLBase.EnsembleAlgorithm
    precision::Symbol
    seed::UInt64
    max_hops::Int
    gap_fp64::Float64
end
EnsembleGB300(precision::Symbol=:fp32; seed=rand(UInt64), max_hops=0, gap_fp64=1e-3) =
    EnsembleGB300(precision, UInt64(seed), max_hops, gap_fp64)

function precision_code(p::Symbol)
    p === :fp64 && return PREC_FP64
    p === :fp32 && return PREC_FP32
    p === :fp32_kahan && return PREC_FP32_KAHAN
    throw(ArgumentError("EnsembleGB300: precision must be :fp64, :fp32 or :fp32_kahan, got $p"))
end

method_name(sim) = nameof(typeof(sim.method))

function method_code(sim)
    ring = sim isa NQCDynamics.RingPolymerSimulation
    m = method_name(sim)
    m === :FSSH && return ring ? METHOD_RPSH : METHOD_FSSH
    m === :AdiabaticIESH && return METHOD_IESH
    m === :DiabaticMDEF && return METHOD_MDEF
    m === :Ehrenfest && !ring && return METHOD_EHRENFEST
    m === :EhrenfestNA && !ring && return METHOD_EHRENFEST_NA
    throw(ArgumentError("EnsembleGB300: $(typeof(sim)) is not supported"))
end

function rescaling_code(sim)
    hasproperty(sim.method, :rescaling) || return Int32(0)
    r = sim.method.rescaling
    r === :standard && return Int32(0)
    r === :vinversion && return Int32(1)
    r === :off && return Int32(2)
    throw(ArgumentError("EnsembleGB300: rescaling $r is not supported"))
end

# Model parameters.  The model types live in NQCModels, which this module
# does not vendor; the field names below are NQCModels' and are the one place
# to adjust if they change.
field(model, names...) = begin
    for n in names
        hasproperty(model, n) && return getproperty(model, n)
    end
    throw(ArgumentError("EnsembleGB300: $(typeof(model)) has none of the fields $(names)"))
end

function model_description(model)
    t = nameof(typeof(model))
    t === :TullyModelOne && return (MODEL_TULLY1, Float64[field(model, :a), field(model, :b), field(model, :c), field(model, :d)], Float64[], Float64[])
    t === :TullyModelTwo && return (MODEL_TULLY2, Float64[field(model, :a), field(model, :b), field(model, :c), field(model, :d), field(model, :e)], Float64[], Float64[])
    t === :TullyModelThree && return (MODEL_TULLY3, Float64[field(model, :a), field(model, :b), field(model, :c)], Float64[], Float64[])
    if t === :SpinBoson
        c = collect(Float64, field(model, :cⱼ, :c))
        w = collect(Float64, field(model, :ωⱼ, :ω))
        return (MODEL_SPINBOSON, Float64[field(model, :ϵ, :eps), field(model, :Δ, :delta)], c, w)
    end
    throw(ArgumentError("EnsembleGB300: model $(typeof(model)) is not supported (the engine's models: Tully 1-3, " *
                        "SpinBoson, AndersonHolstein with the engine's impurities)"))
end

"""Initial conditions of every trajectory through the problem's own `prob_func`
(the reference's Selection and DynamicsVariables), in the C layout."""
function initial_conditions(prob, trajectories::Integer)
    sim = prob.prob.p
    r0 = Float64[]
    v0 = Float64[]
    sre = Float64[]
    sim_ = Float64[]
    state0 = Int32[]
    for i in 1:trajectories
        u = prob.prob_func(deepcopy(prob.prob), i, 1).u0
        append!(r0, vec(NQCDynamics.DynamicsUtils.get_positions(u)))
        append!(v0, vec(NQCDynamics.DynamicsUtils.get_velocities(u)))
        # (nstates, nstates) column-major, as the C layout
        sigma = NQCDynamics.DynamicsUtils.get_quantum_subsystem(u)
        append!(sre, vec(real.(sigma)))
        append!(sim_, vec(imag.(sigma)))
        if method_name(sim) !== :Ehrenfest
            push!(state0, Int32(round(Int, first(u.state)) - 1))
        end
    end
    return r0, v0, sre, sim_, state0
end

output_name(f) = f isa Function ? nameof(f) : nameof(typeof(f))

const FILE_OUTPUTS = (:OutputTotalEnergy, :OutputSurfaceHops, :OutputPosition, :OutputVelocity)

function check_outputs(outputs, file::Bool)
    for f in outputs
        n = output_name(f)
        if file
            n in FILE_OUTPUTS || throw(ArgumentError("EnsembleGB300: FileReduction writes $(FILE_OUTPUTS), not $n"))
        else
            n in (:OutputStateResolvedScattering1D, :PopulationCorrelationFunction, :OutputFinal) ||
                throw(ArgumentError("EnsembleGB300: output $n is not supported"))
        end
    end
end

"""Per-trajectory outputs for FileReduction (reductions.jl:57-91) from the
engine's final state (`nqcd_get_final`): the engine keeps each trajectory at
t0 and t1 only, so `:Time` is `[t0, t1]`, positions and velocities are the
two arrays at those times (stacked by FileReduction on a trailing axis), the
total energy the two values, and the hop count a number."""
function file_batch(h, outputs, t0, t1, shape, r0, v0, trajectories)
    k = prod(shape)
    r = zeros(k * trajectories)
    v = zeros(k * trajectories)
    nh = zeros(Int32, trajectories)
    en = zeros(2 * trajectories)
    GC.@preserve r v nh en check(h, ccall(sym(:nqcd_get_final), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32},
         Ptr{Int32}, Ptr{Float64}),
        h, pointer(r), pointer(v), C_NULL, C_NULL, C_NULL, pointer(nh), C_NULL, C_NULL, pointer(en)))
    block(x, i) = reshape(x[(i - 1) * k + 1:i * k], shape)
    batch = Dictionary{Symbol,Any}[]
    for i in 1:trajectories
        d = Dictionary{Symbol,Any}([:Time], [[t0, t1]])
        for f in outputs
            n = output_name(f)
            n === :OutputTotalEnergy && insert!(d, n, en[2i - 1:2i])
            n === :OutputSurfaceHops && insert!(d, n, Int(nh[i]))
            n === :OutputPosition && insert!(d, n, [block(r0, i), block(r, i)])
            n === :OutputVelocity && insert!(d, n, [block(v0, i), block(v, i)])
        end
        push!(batch, d)
    end
    return batch
end

function SciMLBase.__solve(prob::SciMLBase.AbstractEnsembleProblem,
                           alg::Union{SciMLBase.AbstractDEAlgorithm,Nothing}, ens::EnsembleGB300;
                           trajectories::Integer, dt, saveat=nothing, callback=nothing, kwargs...)
    sim = prob.prob.p
    isnothing(callback) || throw(ArgumentError("EnsembleGB300: callbacks other than |x| > L termination " *
                                               "(given through the engine's terminate_x) are not supported"))
    reduction = prob.reduction
    mean = reduction isa NQCDynamics.Ensembles.MeanReduction
    file = reduction isa NQCDynamics.Ensembles.FileReduction
    mean || file || reduction isa NQCDynamics.Ensembles.SortByTrajectoryReduction ||
        throw(ArgumentError("EnsembleGB300: reduction $(typeof(reduction)) is not supported"))
    outputs = prob.output_func.functions
    check_outputs(outputs, file)
    method = method_code(sim)
    method in (METHOD_FSSH, METHOD_RPSH, METHOD_EHRENFEST) ||
        throw(ArgumentError("EnsembleGB300: this binding marshals the two-state models; IESH and MDEF use " *
                            "nqcd_create with models 20/21 (see INTEGRATION.md)"))
    model, params, bath_a, bath_b = model_description(sim.cache.model)
    t0, t1 = prob.prob.tspan
    stride = isnothing(saveat) ? 0 : round(Int, saveat / dt)
    keep = Any[]
    ring = sim isa NQCDynamics.RingPolymerSimulation
    nbeads = ring ? length(sim.beads) : 0
    natoms = length(sim.atoms.masses)
    ndofs = size(NQCDynamics.DynamicsUtils.get_positions(prob.prob.u0), 1)
    cfg = config(; method, model, ndofs, natoms, nstates=2, params, masses=sim.atoms.masses, keep,
                 precision=precision_code(ens.precision), rescaling=rescaling_code(sim), nbeads_max=nbeads,
                 bath_a, bath_b, beta=ring ? 1.0 / NQCDynamics.get_temperature(sim) : 0.0,
                 ntraj_max=trajectories, init_kind=INIT_GIVEN, save_stride=stride, max_hops=ens.max_hops,
                 gap_fp64=ens.gap_fp64)
    r0, v0, sre, sim_, state0 = initial_conditions(prob, trajectories)
    nsave = stride > 0 ? fld(round(Int, (t1 - t0) / dt), stride) + 1 : 0
    scattering = zeros(2 * 2)
    popcorr = zeros(max(nsave, 1) * 4)
    batch = nothing
    wall = @elapsed begin
        h = GC.@preserve keep create(cfg)
        try
            nb = ring ? fill(Int32(nbeads), trajectories) : Int32[]
            st = isempty(state0) ? Ptr{Int32}(C_NULL) : pointer(state0)
            nbp = isempty(nb) ? Ptr{Int32}(C_NULL) : pointer(nb)
            GC.@preserve r0 v0 sre sim_ state0 nb check(h, ccall(sym(:nqcd_set_initial), Cint,
                (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Int32}),
                h, trajectories, pointer(r0), pointer(v0), pointer(sre), pointer(sim_), st, nbp))
            out = Ref(NqcdOutputs(pointer(scattering), nsave > 0 ? pointer(popcorr) : Ptr{Float64}(C_NULL),
                                  Ptr{Float64}(C_NULL), Int32(0), Int32(0)))
            stats = Ref(zero_stats())
            GC.@preserve scattering popcorr check(h, ccall(sym(:nqcd_run), Cint,
                (Ptr{Cvoid}, Float64, Float64, Float64, UInt64, Ref{NqcdOutputs}, Ref{NqcdStats}),
                h, t0, t1, dt, ens.seed, out, stats))
            LAST_STATS[] = stats[]
            if file
                shape = size(NQCDynamics.DynamicsUtils.get_positions(prob.prob.u0))
                batch = file_batch(h, outputs, t0, t1, shape, r0, v0, trajectories)
            end
        finally
            destroy(h)
        end
    end
    if file
        # the reference's own FileReduction writes the HDF5 groups
        message, _ = reduction(nothing, batch, 1:trajectories)
        return SciMLBase.EnsembleSolution(message, wall, true)
    end
    times = stride > 0 ? collect(range(t0, step=stride * dt, length=nsave)) : [t0, t1]
    result = Dictionary{Symbol,Any}([:Time], [times])
    for f in outputs
        n = output_name(f)
        if n === :OutputStateResolvedScattering1D
            # C layout [2][nstates]: reflection row, then transmission row
            insert!(result, n, (reflection=scattering[1:2], transmission=scattering[3:4]))
        elseif n === :PopulationCorrelationFunction
            # C layout [nsave][2][2] row-major -> one 2x2 matrix per save point
            insert!(result, n, [permutedims(reshape(popcorr[4k+1:4k+4], 2, 2)) for k in 0:(nsave - 1)])
        end
    end
    return SciMLBase.EnsembleSolution(mean ? result : [result], wall, true)
end

"""Engine statistics (`nqcd_stats`) of the last `EnsembleGB300` solve."""
const LAST_STATS = Ref(zero_stats())

end # module NQCDGPU
