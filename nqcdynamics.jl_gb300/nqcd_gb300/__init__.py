"""GB300 ensemble trajectory engine for NQCDynamics.jl's hot path (FSSH, RPSH,
IESH and MDEF ensembles).

The compute runs in libnqcd_gb300.so (CUDA, sm_103a) behind the C ABI of
include/nqcd_gpu.h; this package is the host-side mirror of the reference's
ensemble interface (see api.py) plus the ctypes binding (_lib.py).
"""
from . import _lib
from .api import (
    AdiabaticIESH,
    AdsorbateMetal3D,
    AndersonHolstein,
    DiabaticMDEF,
    DisplacedHarmonic,
    FermiDiracState,
    FileReduction,
    GaussianBroadening,
    OutputImpurityPopulation,
    OutputKineticEnergy,
    OutputPosition,
    OutputVelocity,
    OutputPotentialEnergy,
    ShenviGaussLegendre,
    TrapezoidalRule,
    Adiabatic,
    Atoms,
    Diabatic,
    DecoherenceCorrectionEDC,
    DynamicalDistribution,
    EhrenfestNA,
    Ehrenfest,
    EnsembleGB300,
    EnsembleSerial,
    EnsembleThreads,
    FSSH,
    MeanReduction,
    Normal,
    Uniform,
    OhmicSpectralDensity,
    OutputFinal,
    OutputStateResolvedScattering1D,
    OutputSurfaceHops,
    OutputTotalEnergy,
    PopulationCorrelationFunction,
    PositionHarmonicWigner,
    PureState,
    RingPolymerSimulation,
    Simulation,
    SpinBoson,
    SumReduction,
    TullyModelOne,
    TullyModelThree,
    TullyModelTwo,
    VelocityHarmonicWigner,
    run_dynamics,
)
from ._lib import EngineError, EngineUnavailable

__all__ = [n for n in dir() if not n.startswith("_")]
