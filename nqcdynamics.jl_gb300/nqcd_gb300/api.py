"""Host-side mirror of NQCDynamics.jl's ensemble interface for the GPU engine.

Names, argument meanings and error behaviour follow the reference:

  Atoms, TullyModelOne/Two/Three, SpinBoson + OhmicSpectralDensity   (NQCModels / NQCBase)
  Simulation[FSSH](atoms, model; rescaling)       src/simulations.jl:12-44, fssh.jl:38-45
  Simulation[Ehrenfest](atoms, model)             EhrenfestMethods/ehrenfest.jl:39-41
  RingPolymerSimulation[FSSH](atoms, model, n_beads; temperature)   simulations.jl:46-73, rpsh.jl:5-7
  Simulation[DiabaticMDEF](atoms, model; friction_method, temperature)   mdef.jl:79-100
  Simulation[AdiabaticIESH](atoms, model; rescaling, estimate_probability)   iesh.jl:72-87
  Simulation[EhrenfestNA](atoms, model)           EhrenfestMethods/ehrenfest_na.jl:30-32
  RingPolymerSimulation[DiabaticMDEF](atoms, model, n_beads; friction_method, temperature)   rpmdef.jl:5-27
  RingPolymerSimulation[AdiabaticIESH](atoms, model, n_beads; rescaling, temperature)   rpiesh.jl:3-18
  AndersonHolstein(impurity, bath; coupling, fermi_level, nelectrons),
  TrapezoidalRule, ShenviGaussLegendre, GaussianBroadening      (NQCModels, NQCCalculators)
  FermiDiracState(fermi_level, temperature; statetype)          (NQCDistributions)
  PureState(state, Adiabatic()/Diabatic()), DynamicalDistribution,
  PositionHarmonicWigner / VelocityHarmonicWigner, Normal, Uniform  (NQCDistributions, Distributions)
  OutputStateResolvedScattering1D, OutputSurfaceHops, OutputFinal,
  OutputTotalEnergy                                         src/DynamicsOutputs.jl
  PopulationCorrelationFunction(sim, Diabatic())            src/TimeCorrelationFunctions.jl:61-88
  MeanReduction, SumReduction                               src/Ensembles/reductions.jl:8-52
  run_dynamics(sim, tspan, distribution; trajectories, output, reduction,
               ensemble_algorithm, dt, saveat)              src/Ensembles/run_dynamics.jl:42-136

States are 1-based here, as in Julia; the C ABI is 0-based.  The only
ensemble algorithm is EnsembleGB300: SciMLBase's CPU algorithms raise,
because this engine has no CPU path.
"""
from __future__ import annotations

import os

import math
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import _lib as L

# ---------------------------------------------------------------------------
# Atoms and models
# ---------------------------------------------------------------------------


class Atoms:
    """Atoms(masses) or Atoms(mass) for one atom (NQCBase.Atoms)."""

    def __init__(self, masses):
        m = np.atleast_1d(np.asarray(masses, dtype=np.float64))
        if m.ndim != 1 or len(m) == 0 or np.any(m <= 0):
            raise ValueError("masses must be a non-empty vector of positive numbers")
        self.masses = m

    def __len__(self):
        return len(self.masses)


class Model:
    nstates = 2
    ndofs = 1
    kind: int
    params: tuple


@dataclass
class TullyModelOne(Model):
    a: float = 0.01
    b: float = 1.6
    c: float = 0.005
    d: float = 1.0
    kind = L.MODEL_TULLY1

    @property
    def params(self):
        return (self.a, self.b, self.c, self.d)


@dataclass
class TullyModelTwo(Model):
    a: float = 0.1
    b: float = 0.28
    c: float = 0.015
    d: float = 0.06
    e0: float = 0.05
    kind = L.MODEL_TULLY2

    @property
    def params(self):
        return (self.a, self.b, self.c, self.d, self.e0)


@dataclass
class TullyModelThree(Model):
    a: float = 6e-4
    b: float = 0.1
    c: float = 0.9
    kind = L.MODEL_TULLY3

    @property
    def params(self):
        return (self.a, self.b, self.c)


@dataclass
class OhmicSpectralDensity:
    """J(w) = pi/2 alpha w exp(-w/wc), discretised as
    w_j = -wc ln(1 - j/(N+1)), c_j = sqrt(alpha wc/(N+1)) w_j
    (docs/src/NQCModels/systembathmodels.md:45-59)."""

    ωᶜ: float
    α: float

    def discretise(self, n: int):
        j = np.arange(1, n + 1, dtype=np.float64)
        w = -self.ωᶜ * np.log(1.0 - j / (1 + n))
        c = np.sqrt(self.α * self.ωᶜ / (n + 1)) * w
        return w, c


class SpinBoson(Model):
    """SpinBoson(density, N, ϵ, Δ): V = [[ϵ + c.R, Δ], [Δ, -ϵ - c.R]] + R^T Ω^2 R / 2."""

    kind = L.MODEL_SPINBOSON

    def __init__(self, density: OhmicSpectralDensity, N: int, ϵ: float, Δ: float):
        self.density = density
        self.N = int(N)
        self.ϵ = float(ϵ)
        self.Δ = float(Δ)
        self.ωⱼ, self.cⱼ = density.discretise(self.N)

    @property
    def params(self):
        return (self.ϵ, self.Δ)


# --- metal surfaces (AndersonHolstein) ---------------------------------------


@dataclass
class TrapezoidalRule:
    """M evenly spaced bath levels on [bandmin, bandmax], weights de
    (docs/src/NQCModels/systembathmodels.md:204-214)."""

    M: int
    bandmin: float
    bandmax: float

    def discretise(self):
        from . import workload as WL

        return WL.trapezoidal_rule(self.M, self.bandmin, self.bandmax)


@dataclass
class ShenviGaussLegendre:
    """Gauss-Legendre halves below and above the Fermi level
    (docs/src/NQCModels/systembathmodels.md:241-256)."""

    M: int
    bandmin: float
    bandmax: float

    def discretise(self, fermi_level=0.0):
        from . import workload as WL

        return WL.shenvi_gauss_legendre(self.M, self.bandmin, self.bandmax, fermi_level)


@dataclass
class DisplacedHarmonic:
    """One-dimensional impurity: U0 = k x^2 / 2, U1 = k (x - g)^2 / 2 + delta
    (the adsorbate of the MDEF benchmark configuration)."""

    k: float
    g: float
    delta: float
    ndofs = 1


@dataclass
class AdsorbateMetal3D:
    """One atom in three dimensions above the metal:
    U0 = kxy (x^2 + y^2)/2 + A exp(-a z), h = U1 - U0 = delta - B exp(-b z)
    (the adsorbate of the IESH benchmark configuration)."""

    kxy: float
    A: float
    a: float
    delta: float
    B: float
    b: float
    ndofs = 3


class AndersonHolstein(Model):
    """AndersonHolstein(impurity, bath; coupling, fermi_level, nelectrons):
    impurity state coupled to bath levels e_k with V_k = coupling sqrt(w_k);
    nstates = M + 1 (NQCModels AndersonHolstein, iesh.md:73)."""

    def __init__(self, impurity, bath, coupling: float = 0.02, fermi_level: float = 0.0, nelectrons: int | None = None):
        self.impurity = impurity
        self.bath = bath
        self.fermi_level = float(fermi_level)
        eps, w = bath.discretise(self.fermi_level) if isinstance(bath, ShenviGaussLegendre) else bath.discretise()
        self.eps = np.ascontiguousarray(eps, dtype=np.float64)
        self.V = np.ascontiguousarray(coupling * np.sqrt(w), dtype=np.float64)
        self.nstates = len(self.eps) + 1
        self.nelectrons = self.nstates // 2 if nelectrons is None else int(nelectrons)
        self.ndofs = impurity.ndofs
        if isinstance(impurity, DisplacedHarmonic):
            self.kind = L.MODEL_NEWNS_ANDERSON
        elif isinstance(impurity, AdsorbateMetal3D):
            self.kind = L.MODEL_NEWNS_ANDERSON_3D
        else:
            raise NotImplementedError("impurity model not on the GPU path")


@dataclass
class GaussianBroadening:
    """Friction from the Gaussian-broadened golden rule, width sigma
    (docs/src/NQCModels/frictionmodels.md:91-96)."""

    σ: float


# ---------------------------------------------------------------------------
# Methods and simulations
# ---------------------------------------------------------------------------


@dataclass
class FSSH:
    rescaling: str = "standard"

    def __post_init__(self):
        if self.rescaling not in L.RESCALE:
            raise ValueError(f"rescaling {self.rescaling!r} not recognised (standard, vinversion, off)")


class Ehrenfest:
    """Mean-field (Ehrenfest) dynamics on a two-state model (ehrenfest.jl):
    the FSSH integrator with the force of the density matrix and no hops."""


class DiabaticMDEF:
    """Electronic friction Langevin dynamics on a diabatic model (mdef.jl)."""


class EhrenfestNA:
    """Mean-field dynamics of independent electrons in a metal
    (ehrenfest_na.jl): the IESH integrator with the force of the orbitals."""


@dataclass
class DecoherenceCorrectionEDC:
    """Energy-based decoherence correction (decoherence_corrections.jl:8-13)."""

    C: float = 0.1


@dataclass
class AdiabaticIESH:
    """Independent-electron surface hopping (iesh.jl:72-87)."""

    rescaling: str = "standard"
    estimate_probability: bool = True
    decoherence: Any = None  # None (DecoherenceCorrectionNone) or DecoherenceCorrectionEDC

    def __post_init__(self):
        if self.rescaling not in L.RESCALE:
            raise ValueError(f"rescaling {self.rescaling!r} not recognised (standard, vinversion, off)")


class _MethodIndexed(type):
    def __getitem__(cls, method):
        def make(*args, **kwargs):
            return cls(*args, method=method, **kwargs)

        return make


class Simulation(metaclass=_MethodIndexed):
    """Simulation[FSSH](atoms, model; rescaling=:standard)."""

    def __init__(self, atoms: Atoms, model: Model, method=FSSH, rescaling: str = "standard", temperature=0.0,
                 friction_method=None, estimate_probability: bool = True, decoherence=None):
        self.atoms = atoms
        self.model = model
        self.temperature = float(temperature)
        if method is DiabaticMDEF:
            if not isinstance(model, AndersonHolstein):
                raise NotImplementedError("DiabaticMDEF runs on AndersonHolstein(DisplacedHarmonic(...) or "
                                          "AdsorbateMetal3D(...), bath)")
            if not isinstance(friction_method, GaussianBroadening):
                raise ValueError("DiabaticMDEF needs friction_method=GaussianBroadening(sigma)")
            if not temperature > 0:
                raise ValueError("MDEF needs a positive temperature")
            if len(atoms) != 1:
                raise ValueError("one adsorbate atom with one degree of freedom")
            self.method = DiabaticMDEF()
            self.friction_method = friction_method
            return
        if method is AdiabaticIESH or method is EhrenfestNA:
            if not isinstance(model, AndersonHolstein) or model.kind != L.MODEL_NEWNS_ANDERSON_3D:
                raise NotImplementedError(f"{method.__name__} runs on AndersonHolstein(AdsorbateMetal3D(...), bath)")
            if len(atoms) != 1:
                raise ValueError("one adsorbate atom with three degrees of freedom")
            if decoherence is not None and not isinstance(decoherence, DecoherenceCorrectionEDC):
                raise NotImplementedError("decoherence: DecoherenceCorrectionEDC or None")
            self.method = AdiabaticIESH(rescaling, estimate_probability, decoherence) if method is AdiabaticIESH \
                else EhrenfestNA()
            return
        if method is Ehrenfest:
            self.method = Ehrenfest()
        elif method is FSSH:
            self.method = FSSH(rescaling)
        else:
            raise NotImplementedError(f"method {method} is not on the GPU path")
        if isinstance(model, SpinBoson):
            if len(atoms) != model.N:
                raise ValueError("SpinBoson needs one atom per bath mode")
        elif len(atoms) != 1:
            raise ValueError("Tully models have one atom with one degree of freedom")

    @property
    def size(self):
        return (self.model.ndofs, len(self.atoms))

    @property
    def ndof(self):
        return self.model.ndofs * len(self.atoms)


class RingPolymerSimulation(metaclass=_MethodIndexed):
    """RingPolymerSimulation[FSSH](atoms, model, n_beads; temperature),
    RingPolymerSimulation[DiabaticMDEF](atoms, model, n_beads; friction_method,
    temperature) (rpmdef.jl:5-27) and
    RingPolymerSimulation[AdiabaticIESH](atoms, model, n_beads; rescaling,
    estimate_probability, temperature) (rpiesh.jl:3-18)."""

    def __init__(self, atoms: Atoms, model: Model, n_beads, method=FSSH, rescaling: str = "standard",
                 temperature: float = 0.0, friction_method=None, estimate_probability: bool = True,
                 decoherence=None):
        if method is AdiabaticIESH:
            if not isinstance(model, AndersonHolstein) or model.kind != L.MODEL_NEWNS_ANDERSON_3D:
                raise NotImplementedError("ring-polymer IESH runs on AndersonHolstein(AdsorbateMetal3D(...), bath)")
            if decoherence is not None:
                raise NotImplementedError("ring-polymer IESH runs without decoherence correction")
            if not temperature > 0:
                raise ValueError("ring polymers need a positive temperature")
            if len(atoms) != 1 or not 2 <= int(n_beads) <= 32:
                raise ValueError("one adsorbate atom with three degrees of freedom and 2..32 beads")
            self.atoms, self.model = atoms, model
            self.method = AdiabaticIESH(rescaling, estimate_probability, None)
            self.temperature = float(temperature)
            self.n_beads = int(n_beads)
            return
        if method is DiabaticMDEF:
            if not isinstance(model, AndersonHolstein) or model.kind != L.MODEL_NEWNS_ANDERSON:
                raise NotImplementedError("ring-polymer MDEF runs on AndersonHolstein(DisplacedHarmonic(...), bath)")
            if not isinstance(friction_method, GaussianBroadening):
                raise ValueError("DiabaticMDEF needs friction_method=GaussianBroadening(sigma)")
            if not temperature > 0:
                raise ValueError("ring polymers need a positive temperature")
            if len(atoms) != 1 or not 2 <= int(n_beads) <= 32:
                raise ValueError("one adsorbate degree of freedom and 2..32 beads")
            self.atoms, self.model, self.method = atoms, model, DiabaticMDEF()
            self.friction_method = friction_method
            self.temperature = float(temperature)
            self.n_beads = int(n_beads)
            return
        if method is not FSSH:
            raise NotImplementedError(f"method {method} is not on the GPU path")
        if isinstance(model, SpinBoson) or len(atoms) != 1:
            raise NotImplementedError("ring-polymer surface hopping runs on the one-dimensional Tully models")
        if not temperature > 0:
            raise ValueError("ring polymers need a positive temperature")
        self.atoms = atoms
        self.model = model
        self.method = FSSH(rescaling)
        self.temperature = float(temperature)
        self.n_beads = n_beads

    @property
    def beta(self):
        return 1.0 / self.temperature


# ---------------------------------------------------------------------------
# Distributions
# ---------------------------------------------------------------------------


class Adiabatic:
    pass


class Diabatic:
    pass


@dataclass
class PureState:
    state: int
    statetype: Any = field(default_factory=Diabatic)

    def init_kind(self):
        return L.INIT_ADIABATIC_PURE if isinstance(self.statetype, Adiabatic) else L.INIT_DIABATIC_PURE


@dataclass
class PositionHarmonicWigner:
    """Wigner position distribution of a harmonic oscillator (hbar = 1)."""

    ω: float
    β: float
    m: float

    def sigma(self):
        return math.sqrt(1.0 / (2.0 * self.m * self.ω * math.tanh(self.β * self.ω / 2.0)))

    def sampler(self):
        return (L.SAMPLE_NORMAL, 0.0, self.sigma())


@dataclass
class VelocityHarmonicWigner:
    ω: float
    β: float
    m: float

    def sigma(self):
        return math.sqrt(self.ω / (2.0 * self.m * math.tanh(self.β * self.ω / 2.0)))

    def sampler(self):
        return (L.SAMPLE_NORMAL, 0.0, self.sigma())


@dataclass
class Normal:
    """Distributions.Normal(mean, std) for one degree of freedom."""

    mean: float = 0.0
    std: float = 1.0

    def sigma(self):
        return self.std

    def sampler(self):
        return (L.SAMPLE_NORMAL, self.mean, self.std)


@dataclass
class Uniform:
    """Distributions.Uniform(a, b) for one degree of freedom."""

    a: float = 0.0
    b: float = 1.0

    def sampler(self):
        return (L.SAMPLE_UNIFORM, self.a, self.b)


class DynamicalDistribution:
    """DynamicalDistribution(velocity, position, size): each of velocity and
    position is a scalar, an array of per-dof samplers/values, or a sequence
    of explicit samples (one per trajectory)."""

    def __init__(self, velocity, position, size):
        self.velocity = velocity
        self.position = position
        self.size = tuple(size)

    def __mul__(self, other):
        return ProductDistribution(self, other)

    def samplers(self, which):
        """Per-dof (kind, a, b) triples for device-side sampling
        (nqcd_sample_initial), or ValueError if the specification holds
        explicit per-trajectory samples."""
        spec = self.velocity if which == "v" else self.position
        n = int(np.prod(self.size))
        if hasattr(spec, "sampler"):
            return [spec.sampler()] * n
        flat = list(np.asarray(spec, dtype=object).reshape(-1, order="F"))
        if len(flat) == 1 and not hasattr(flat[0], "sampler"):
            return [(L.SAMPLE_FIXED, float(flat[0]), 0.0)] * n
        if len(flat) == n:
            return [s.sampler() if hasattr(s, "sampler") else (L.SAMPLE_FIXED, float(s), 0.0) for s in flat]
        raise ValueError("explicit per-trajectory samples cannot be drawn on the device")

    def sample(self, which, ntraj, rng):
        spec = self.velocity if which == "v" else self.position
        n = int(np.prod(self.size))
        if hasattr(spec, "sampler"):
            spec = [spec] * n
        if isinstance(spec, (list, tuple)) or (isinstance(spec, np.ndarray) and spec.dtype == object):
            flat = list(np.asarray(spec, dtype=object).reshape(-1, order="F"))
            if len(flat) == n and any(hasattr(s, "sampler") for s in flat):
                out = np.empty((ntraj, n))
                for d, s in enumerate(flat):
                    kind, a, b = s.sampler() if hasattr(s, "sampler") else (L.SAMPLE_FIXED, float(s), 0.0)
                    if kind == L.SAMPLE_FIXED:
                        out[:, d] = a
                    elif kind == L.SAMPLE_UNIFORM:
                        out[:, d] = a + (b - a) * rng.random(ntraj)
                    else:
                        out[:, d] = a + b * rng.standard_normal(ntraj)
                return out
        arr = np.asarray(spec, dtype=np.float64)
        if arr.size == 1:
            return np.full((ntraj, n), float(arr))
        if arr.shape == self.size or arr.size == n:
            return np.broadcast_to(arr.reshape(-1, order="F"), (ntraj, n)).copy()
        if arr.shape == (ntraj,) + tuple(self.size):  # one Julia-shaped array per trajectory: column-major
            return arr.transpose(0, *range(arr.ndim - 1, 0, -1)).reshape(ntraj, -1).copy()
        if arr.ndim >= 1 and arr.shape[0] == ntraj:
            return arr.reshape(ntraj, -1).copy()
        raise ValueError("cannot interpret distribution specification")


@dataclass
class FermiDiracState:
    """FermiDiracState(fermi_level, temperature; statetype=Adiabatic()):
    occupations sampled at the temperature (atomic units of energy)."""

    fermi_level: float
    temperature: float
    statetype: Any = field(default_factory=Adiabatic)

    def __post_init__(self):
        if not isinstance(self.statetype, Adiabatic):
            raise NotImplementedError("the GPU path samples adiabatic occupations")

    @property
    def β(self):
        return 1.0 / self.temperature


@dataclass
class ProductDistribution:
    nuclear: DynamicalDistribution
    electronic: Any


# ---------------------------------------------------------------------------
# Outputs and reductions
# ---------------------------------------------------------------------------


@dataclass
class OutputStateResolvedScattering1D:
    sim: Any
    type: str = "adiabatic"

    def __post_init__(self):
        if self.type not in ("adiabatic",):
            raise ValueError(f"{self.type} not recognised: the GPU path evaluates adiabatic populations")


@dataclass
class PopulationCorrelationFunction:
    sim: Any
    statetype: Any = field(default_factory=Diabatic)

    def __post_init__(self):
        if not isinstance(self.statetype, Diabatic):
            raise NotImplementedError("the GPU path evaluates the diabatic population correlation")


class OutputFinal:
    pass


class OutputSurfaceHops:
    pass


class OutputTotalEnergy:
    pass


class OutputKineticEnergy:
    pass


class OutputPotentialEnergy:
    pass


class OutputPosition:
    pass


class OutputVelocity:
    pass


class OutputImpurityPopulation:
    """IESH: population of the impurity state, row 0 of
    iesh_diabatic_population (iesh.jl:351-369), at each save point."""


class MeanReduction:
    pass


class SumReduction:
    pass


class SortByTrajectoryReduction:
    pass


class FileReduction:
    """Per-trajectory outputs written to a file, as FileReduction does
    (src/Ensembles/reductions.jl:57-91): one group `trajectory_<id>` per
    trajectory (ids from 1) holding one array per output name, `Time`
    included.  This image has no HDF5 library, so the container is NumPy's
    .npz with the same paths (`trajectory_3/OutputTotalEnergy`), and the file
    name takes the .npz extension where the reference's takes .h5.  Outputs
    that are numbers or arrays per trajectory are written (total energy and
    positions or velocities at the engine's time points, t0 and t1; hop
    counts); others raise, as the reference's does for outputs it cannot
    convert."""

    def __init__(self, filename: str):
        root, ext = os.path.splitext(filename)
        self.filename = filename if ext == ".npz" else root + ".npz"

    def write(self, times, per_traj: dict) -> str:
        n = len(next(iter(per_traj.values())))
        arrays = {}
        for i in range(n):
            g = f"trajectory_{i + 1}"
            arrays[f"{g}/Time"] = np.asarray(times, np.float64)
            for name, arr in per_traj.items():
                arrays[f"{g}/{name}"] = np.asarray(arr[i])
        np.savez(self.filename, **arrays)
        return f"Output written to {self.filename}."


# ---------------------------------------------------------------------------
# Ensemble algorithms
# ---------------------------------------------------------------------------


class EnsembleSerial:
    pass


class EnsembleThreads:
    pass


@dataclass
class EnsembleGB300:
    """GPU ensemble algorithm: precision 'fp64' (plain, bit-identical to the
    FP64 reference integration), 'fp32' (fast path, FP64 accumulation of
    positions and velocities) or 'fp32_kahan' (fast path, compensated FP32
    accumulation)."""

    precision: str = "fp64"
    gap_fp64: float = 1e-3
    max_hops: int = 16
    seed: int = 20261203
    friction_surrogate: Any = None  # MDEF: (weights, meta) of a trained network, or None
    exact_friction_every: int = 0   # MDEF surrogate: judge the network against the exact friction every k steps
    surrogate_tolerance: float = 0.1  # judged relative error that retires the network for a trajectory
    device_sampling: bool = False   # draw the nuclear initial conditions on the GPU (nqcd_sample_initial)


# ---------------------------------------------------------------------------
# run_dynamics
# ---------------------------------------------------------------------------


def _output_name(o):
    return o.__name__ if isinstance(o, type) else type(o).__name__


def build_config(sim, electronic: PureState, ntraj: int, alg: EnsembleGB300, save_stride: int):
    model = sim.model
    cfg = L.nqcd_config()
    ehrenfest = isinstance(sim.method, Ehrenfest)
    cfg.method = L.METHOD_EHRENFEST if ehrenfest else L.METHOD_FSSH
    cfg.model = model.kind
    cfg.precision = {"fp64": L.PREC_FP64, "fp32": L.PREC_FP32, "fp32_kahan": L.PREC_FP32_KAHAN}[alg.precision]
    cfg.rescaling = 0 if ehrenfest else L.RESCALE[sim.method.rescaling]
    cfg.ndofs = model.ndofs
    cfg.natoms = len(sim.atoms)
    cfg.nstates = model.nstates
    params = np.asarray(model.params, dtype=np.float64)
    masses = np.ascontiguousarray(sim.atoms.masses, dtype=np.float64)
    keep = [params, masses]
    cfg.nparams = len(params)
    cfg.params = L.dptr(params)
    if isinstance(model, SpinBoson):
        c = np.ascontiguousarray(model.cⱼ)
        w = np.ascontiguousarray(model.ωⱼ)
        keep += [c, w]
        cfg.nbath = model.N
        cfg.bath_a = L.dptr(c)
        cfg.bath_b = L.dptr(w)
    cfg.masses = L.dptr(masses)
    cfg.ntraj_max = ntraj
    if not (1 <= electronic.state <= model.nstates):
        raise ValueError("PureState index outside 1..nstates")
    cfg.init_kind = electronic.init_kind()
    cfg.init_state = electronic.state - 1
    cfg.save_stride = save_stride
    cfg.max_hops = alg.max_hops
    cfg.gap_fp64 = alg.gap_fp64
    return cfg, keep


def run_dynamics(sim, tspan, distribution, *, output, trajectories: int = 1, reduction=None,
                 ensemble_algorithm=None, dt: float = 1.0, saveat=None, seed: int | None = None,
                 rng: np.random.Generator | None = None):
    """Run an ensemble through the GPU engine and reduce the outputs.

    Returns a dict keyed like the reference's MeanReduction Dictionary
    (:Time plus one entry per output) or, for one trajectory, that
    trajectory's outputs."""
    alg = ensemble_algorithm if ensemble_algorithm is not None else EnsembleGB300()
    if isinstance(alg, (EnsembleSerial, EnsembleThreads)) or alg in (EnsembleSerial, EnsembleThreads):
        raise NotImplementedError("this engine has no CPU path: use ensemble_algorithm=EnsembleGB300()")
    if not isinstance(alg, EnsembleGB300):
        raise TypeError("ensemble_algorithm must be EnsembleGB300")
    if isinstance(sim, RingPolymerSimulation):
        if isinstance(sim.method, (DiabaticMDEF, AdiabaticIESH)):
            return _run_metal(sim, tspan, distribution, output, trajectories, reduction, alg, dt, saveat, seed, rng)
        raise NotImplementedError("ring-polymer surface hopping runs through run_ring_polymer_ensemble")
    if isinstance(getattr(sim, "method", None), (DiabaticMDEF, AdiabaticIESH, EhrenfestNA)):
        return _run_metal(sim, tspan, distribution, output, trajectories, reduction, alg, dt, saveat, seed, rng)
    if not isinstance(distribution, ProductDistribution):
        raise TypeError("distribution must be DynamicalDistribution * PureState")
    outputs = output if isinstance(output, (tuple, list)) else (output,)
    reduction = reduction if reduction is not None else MeanReduction()
    if not isinstance(reduction, (MeanReduction, SumReduction, FileReduction)):
        raise NotImplementedError("the GPU path reduces on the device (MeanReduction, SumReduction) or writes "
                                  "per-trajectory outputs (FileReduction)")
    t0, t1 = float(tspan[0]), float(tspan[1])
    save_stride = 0
    for o in outputs:
        if isinstance(o, PopulationCorrelationFunction):
            if saveat is None:
                raise ValueError("PopulationCorrelationFunction needs saveat")
            stride = float(saveat) / dt
            if abs(stride - round(stride)) > 1e-9 or round(stride) < 1:
                raise ValueError("saveat must be a positive multiple of dt on the GPU path")
            save_stride = int(round(stride))
    ntraj = int(trajectories)
    seed_ = alg.seed if seed is None else seed
    if alg.device_sampling:
        pos, vel = distribution.nuclear.samplers("r"), distribution.nuclear.samplers("v")
    else:
        rng = rng if rng is not None else np.random.default_rng(seed_)
        r0 = distribution.nuclear.sample("r", ntraj, rng)
        v0 = distribution.nuclear.sample("v", ntraj, rng)
    cfg, keep = build_config(sim, distribution.electronic, ntraj, alg, save_stride)
    eng = L.Engine(cfg, keep)
    try:
        if alg.device_sampling:
            eng.sample_initial(ntraj, pos, vel, seed_)
        else:
            eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0))
        sc = np.zeros(4)
        pc = None
        if save_stride:
            nsteps = int(round((t1 - t0) / dt))
            pc = np.zeros((nsteps // save_stride + 1) * 4 + 4)
        out, stats = eng.run(t0, t1, dt, alg.seed if seed is None else seed, scattering=sc, popcorr=pc)
        if isinstance(reduction, FileReduction):
            final = eng.get_final(sim.ndof)
            start = None if alg.device_sampling else (r0, v0)
            return reduction.write([t0, t1], _per_trajectory(outputs, final, start, hops=True))
        result: dict[str, Any] = {}
        scale = ntraj if isinstance(reduction, SumReduction) else 1
        final = None
        for o in outputs:
            name = _output_name(o)
            if isinstance(o, OutputStateResolvedScattering1D):
                result[name] = {"reflection": sc[:2] * scale, "transmission": sc[2:] * scale}
            elif isinstance(o, PopulationCorrelationFunction):
                result[name] = pc[: out.nsave * 4].reshape(out.nsave, 2, 2) * scale
                result["Time"] = t0 + dt * save_stride * np.arange(out.nsave)
            else:
                if final is None:
                    final = eng.get_final(sim.ndof)
                if o is OutputFinal or isinstance(o, OutputFinal):
                    result["OutputFinal"] = final
                elif o is OutputTotalEnergy or isinstance(o, OutputTotalEnergy):
                    result["OutputTotalEnergy"] = final["energy"]
                elif o is OutputSurfaceHops or isinstance(o, OutputSurfaceHops):
                    result["OutputSurfaceHops"] = final["nhops"]
                else:
                    raise NotImplementedError(f"output {name} is not available on the GPU path")
        result["_stats"] = stats
        return result
    finally:
        eng.close()


def _per_trajectory(outputs, final, start, hops):
    """Per-trajectory arrays of FileReduction at the engine's time points
    (t0, t1): total energy (ntraj, 2), positions and velocities (ntraj, ...,
    2), surface-hop counts."""
    per = {}
    for o in outputs:
        name = _output_name(o)
        if name == "OutputTotalEnergy":
            per[name] = final["energy"]
        elif name == "OutputSurfaceHops" and hops:
            per[name] = final["nhops"]
        elif name in ("OutputPosition", "OutputVelocity") and start is not None:
            key, q = ("r", 0) if name == "OutputPosition" else ("v", 1)
            a = np.asarray(start[q], np.float64).reshape(final[key].shape)
            per[name] = np.stack([a, final[key]], axis=-1)
        else:
            raise TypeError(f"Cannot convert output {name} to the file format")
    if not per:
        raise TypeError("FileReduction needs at least one per-trajectory output")
    return per


def _metal_config(sim, ntraj, alg, save_stride):
    model = sim.model
    mdef = isinstance(sim.method, DiabaticMDEF)
    cfg = L.nqcd_config()
    ena = isinstance(sim.method, EhrenfestNA)
    cfg.method = L.METHOD_MDEF if mdef else (L.METHOD_EHRENFEST_NA if ena else L.METHOD_IESH)
    cfg.model = model.kind
    cfg.precision = {"fp64": L.PREC_FP64, "fp32": L.PREC_FP32}[alg.precision]
    cfg.ndofs, cfg.natoms, cfg.nstates = model.ndofs, 1, model.nstates
    imp = model.impurity
    if mdef:
        if isinstance(imp, AdsorbateMetal3D):  # three coordinates; the friction tensor acts along z
            params = np.array([imp.kxy, imp.A, imp.a, imp.delta, imp.B, imp.b, model.fermi_level,
                               sim.friction_method.σ])
        else:
            params = np.array([imp.k, imp.g, imp.delta, model.fermi_level, sim.friction_method.σ])
        cfg.beta = 1.0 / sim.temperature
        cfg.use_friction_surrogate = int(alg.friction_surrogate is not None)
        cfg.exact_friction_every = alg.exact_friction_every
        cfg.surrogate_tolerance = alg.surrogate_tolerance
    else:
        params = np.array([imp.kxy, imp.A, imp.a, imp.delta, imp.B, imp.b])
        cfg.rescaling = 0 if ena else L.RESCALE[sim.method.rescaling]
        cfg.exact_hop_probability = 0 if ena else int(not sim.method.estimate_probability)
        if not ena and sim.method.decoherence is not None:
            cfg.decoherence_C = sim.method.decoherence.C
        cfg.nelectrons = model.nelectrons
        cfg.max_hops = alg.max_hops
        cfg.gap_fp64 = alg.gap_fp64  # FP32 path: FP64 refinement of near-degenerate roots
    masses = np.ascontiguousarray(sim.atoms.masses, dtype=np.float64)
    cfg.nparams, cfg.params, cfg.masses = len(params), L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(model.eps), L.dptr(model.eps), L.dptr(model.V)
    cfg.ntraj_max = ntraj
    cfg.save_stride = save_stride
    return cfg, [params, masses, model.eps, model.V]


def _run_metal(sim, tspan, distribution, output, trajectories, reduction, alg, dt, saveat, seed, rng):
    """run_dynamics for Simulation[DiabaticMDEF] and Simulation[AdiabaticIESH]."""
    mdef = isinstance(sim.method, DiabaticMDEF)
    outputs = output if isinstance(output, (tuple, list)) else (output,)
    reduction = reduction if reduction is not None else MeanReduction()
    if not isinstance(reduction, (MeanReduction, FileReduction)):
        raise NotImplementedError("the GPU path reduces on the device (MeanReduction) or writes per-trajectory "
                                  "outputs (FileReduction)")
    if mdef:
        nuclear = distribution
        if isinstance(distribution, ProductDistribution):
            raise TypeError("DiabaticMDEF takes a nuclear DynamicalDistribution")
    else:
        if not (isinstance(distribution, ProductDistribution) and isinstance(distribution.electronic, FermiDiracState)):
            raise TypeError("AdiabaticIESH takes DynamicalDistribution * FermiDiracState")
        if abs(distribution.electronic.fermi_level - sim.model.fermi_level) > 1e-12:
            raise ValueError("Fermi level of model and distribution do not match")  # iesh.jl:104-113
        nuclear = distribution.nuclear
    t0, t1 = float(tspan[0]), float(tspan[1])
    timeseries = [o for o in outputs if o in (OutputKineticEnergy, OutputPotentialEnergy, OutputPosition,
                                              OutputImpurityPopulation)
                  or isinstance(o, (OutputKineticEnergy, OutputPotentialEnergy, OutputPosition, OutputImpurityPopulation))]
    save_stride = 0
    if timeseries and not isinstance(reduction, FileReduction):
        if saveat is None:
            raise ValueError("time-series outputs need saveat")
        stride = float(saveat) / dt
        if abs(stride - round(stride)) > 1e-9 or round(stride) < 1:
            raise ValueError("saveat must be a positive multiple of dt on the GPU path")
        save_stride = int(round(stride))
    ntraj = int(trajectories)
    rp = isinstance(sim, RingPolymerSimulation)
    if rp and mdef and save_stride:
        raise NotImplementedError("ring-polymer MDEF reports final states (OutputFinal, OutputTotalEnergy) on the GPU "
                                  "path")
    if rp and not mdef and abs(distribution.electronic.β * sim.temperature - 1.0) > 1e-12:
        raise NotImplementedError("ring-polymer IESH on the GPU path takes the Fermi-Dirac temperature equal to the "
                                  "ring-polymer temperature")
    rng = rng if rng is not None else np.random.default_rng(alg.seed if seed is None else seed)
    r0 = nuclear.sample("r", ntraj, rng)
    v0 = nuclear.sample("v", ntraj, rng)
    cfg, keep = _metal_config(sim, ntraj, alg, save_stride)
    if rp:
        cfg.nbeads_max = sim.n_beads
    if not mdef:
        cfg.beta = distribution.electronic.β
        cfg.init_kind = L.INIT_FERMI_DIRAC
    eng = L.Engine(cfg, keep)
    try:
        if mdef and alg.friction_surrogate is not None:
            eng.mlp_set(*alg.friction_surrogate)
        eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0))
        nsteps = int(round((t1 - t0) / dt))
        obs = np.zeros(((nsteps // save_stride + 1) if save_stride else 1) * 4)
        out, stats = eng.run(t0, t1, dt, alg.seed if seed is None else seed, observables=obs)
        mdef_dofs = sim.n_beads if rp else sim.model.ndofs
        if isinstance(reduction, FileReduction):
            final = eng.get_final(mdef_dofs) if mdef else \
                eng.get_final_iesh(sim.model.nstates, sim.model.nelectrons)
            return reduction.write([t0, t1], _per_trajectory(outputs, final, (r0, v0), hops=not mdef))
        ob = obs[: out.nsave * 4].reshape(out.nsave, 4)
        result: dict[str, Any] = {}
        if save_stride:
            result["Time"] = t0 + dt * save_stride * np.arange(out.nsave)
        final = None
        for o in outputs:
            name = _output_name(o)
            if name == "OutputKineticEnergy":
                result[name] = ob[:, 2] if mdef else ob[:, 1]
            elif name == "OutputPosition":
                result[name] = ob[:, 0]  # MDEF: x (3-D adsorbate: z); IESH: height z
            elif name == "OutputPotentialEnergy" and not mdef:
                result[name] = ob[:, 3]
            elif name == "OutputImpurityPopulation" and not mdef:
                result[name] = ob[:, 2]
            elif name in ("OutputFinal", "OutputTotalEnergy", "OutputSurfaceHops"):
                if final is None:  # ring polymers: r, v (ntraj, nbeads, ...)
                    final = eng.get_final(mdef_dofs) if mdef else \
                        eng.get_final_iesh(sim.model.nstates, sim.model.nelectrons)
                if name == "OutputFinal":
                    result[name] = final
                elif name == "OutputTotalEnergy":
                    result[name] = final["energy"].mean(axis=0)
                elif not mdef:
                    result[name] = final["nhops"].mean()
                else:
                    raise NotImplementedError("DiabaticMDEF has no surface hops")
            else:
                raise NotImplementedError(f"output {name} is not available on the GPU path for this method")
        result["_stats"] = stats
        return result
    finally:
        eng.close()
