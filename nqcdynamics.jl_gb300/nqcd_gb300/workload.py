"""Benchmark workloads (synthetic inputs with the shapes of the reference's
configurations) and the algorithmic work per trajectory-step used for the
roofline.

Spin-boson FSSH (the headline workload): Ohmic bath, 100 discretised modes
(Kondo parameter 0.1, omega_c = 2.5), Delta = 1, eps = 0, beta = 5, unit
masses, Wigner-sampled harmonic positions and velocities, diabatic pure
state 1, dt = 0.05, t in [0, 20] (400 steps), population correlation saved
every 0.1 (201 points), 100 000 trajectories.  The shapes follow the
reference's spin-boson example (docs/src/examples/spinboson.md:20-65) with
the step and Kondo parameter of the benchmark configuration.  No dataset is
involved: inputs are drawn from a seeded generator.
"""
from __future__ import annotations

import numpy as np

SEED = 20261203


def spin_boson_inputs(ntraj: int, nmodes: int = 100, *, wc: float = 2.5, alpha: float = 0.1, beta: float = 5.0,
                      seed: int = SEED, traj_offset: int = 0):
    """Bath frequencies/couplings and Wigner samples (trajectory-major)."""
    j = np.arange(1, nmodes + 1, dtype=np.float64)
    w = -wc * np.log(1.0 - j / (nmodes + 1))
    c = np.sqrt(alpha * wc / (nmodes + 1)) * w
    sx = np.sqrt(1.0 / (2.0 * w * np.tanh(beta * w / 2.0)))
    sv = np.sqrt(w / (2.0 * np.tanh(beta * w / 2.0)))
    rng = np.random.default_rng([seed, traj_offset])
    r0 = rng.standard_normal((ntraj, nmodes)) * sx
    v0 = rng.standard_normal((ntraj, nmodes)) * sv
    return w, c, r0, v0


# ---------------------------------------------------------------------------
# Algorithmic work of the reference algorithm per nuclear step of one
# trajectory (two electronic states), counted operation by operation from
# bab_electronics.jl:61-91 and the files it calls:
#
#  electronics (Tsit5, 5 sub-steps, 31 right-hand-side evaluations):
#    one f! evaluation on complex 2x2 matrices: coupling interpolation
#    (4 entries x 6) + eigenvalue interpolation (2 x 6) + A*(-i) (4 x 6)
#    + two complex 2x2 products (16 complex MACs x 8) + subtraction (8)
#    + times -i (4 x 6) = 220 flops;  31 x 220 = 6820
#    stage combinations: 48 flops per real component per sub-step,
#    8 components, 5 sub-steps = 1920
#  per degree of freedom: B, A, B kicks (6), potential sums (4), derivative
#    (3), Z^T dH Z (21), coupling and force divisions (3), dynamical
#    coupling (8), hop probability (5) = 50
#  eigen-decomposition, hop test and rescaling: 30
# ---------------------------------------------------------------------------
ELECTRONIC_FLOPS_2STATE = 6820 + 1920
PER_DOF_FLOPS = 50
FIXED_FLOPS = 30


def ref_flops_per_traj_step(ndof: int) -> int:
    return ELECTRONIC_FLOPS_2STATE + PER_DOF_FLOPS * ndof + FIXED_FLOPS


def ref_hbm_bytes_per_traj_step(ndof: int) -> int:
    """State that an ideal kernel keeps on chip: 0 bytes per step; the
    per-trajectory input and output (2 ndof doubles each way) is amortised
    over the run and counted per run, not per step."""
    return 0
