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


AU_PER_FS = 41.341373335
KELVIN_AU = 3.166811563e-6


def shenvi_gauss_legendre(M: int, a: float, b: float, ef: float = 0.0):
    """Bath levels and weights of the ShenviGaussLegendre discretisation
    (docs/src/NQCModels/systembathmodels.md:241-256): Gauss-Legendre halves
    below and above the Fermi level (upper shift (ef + b)/2, which maps the
    knots into [ef, b])."""
    x, w = np.polynomial.legendre.leggauss(M // 2)
    lo = 0.5 * (ef - a) * x + 0.5 * (a + ef)
    hi = 0.5 * (b - ef) * x + 0.5 * (ef + b)
    return np.concatenate([lo, hi]), np.concatenate([0.5 * (ef - a) * w, 0.5 * (b - ef) * w])


def newns_anderson_mdef(ntraj: int, *, M: int = 200, coupling: float = 0.02, mass: float = 1837.0,
                        omega: float = 0.004, g: float = 1.0, sigma: float = 0.01, temperature_K: float = 300.0,
                        hot: float = 10.0, seed: int = SEED, traj_offset: int = 0):
    """Electronic-friction workload: one adsorbate degree of freedom (hydrogen
    mass) on a displaced-harmonic impurity coupled to a metal band of M
    Gauss-Legendre states on [-0.5, 0.5] Hartree with V_k = coupling sqrt(w_k),
    Fermi level 0, electronic temperature 300 K.  The impurity level
    h(x) = k g (g/2 - x) + delta with delta = -k g^2 / 2 crosses the Fermi
    level at x = 0.  Initial conditions are thermal at `hot` times the
    electronic temperature (a vibrationally hot adsorbate that the friction
    cools).  Returns the model parameters and initial positions/velocities."""
    eps, w = shenvi_gauss_legendre(M, -0.5, 0.5, 0.0)
    k = mass * omega**2
    T = temperature_K * KELVIN_AU
    rng = np.random.default_rng([seed, traj_offset, 4])
    x0 = rng.standard_normal(ntraj) * np.sqrt(hot * T / k)
    v0 = rng.standard_normal(ntraj) * np.sqrt(hot * T / mass)
    return dict(eps=eps, weights=w, V=coupling * np.sqrt(w), k=k, g=g, delta=-0.5 * k * g * g, mu=0.0, sigma=sigma,
                beta=1.0 / T, mass=mass, x0=x0, v0=v0, dt=0.1 * AU_PER_FS)


EV_AU = 1.0 / 27.211386245988
AMU_AU = 1822.888486


def trapezoidal_rule(M: int, a: float, b: float):
    """Bath levels and squared-coupling weights of TrapezoidalRule
    (docs/src/NQCModels/systembathmodels.md:204-214): M evenly spaced levels
    on [a, b], |V_n|^2 = |V(e)|^2 (b - a) / (M - 1)."""
    eps = a + np.arange(M) * (b - a) / (M - 1)
    return eps, np.full(M, (b - a) / (M - 1))


def newns_anderson_iesh(ntraj: int, *, nstates: int = 80, nelectrons: int = 40, coupling: float = 0.04,
                        mass_amu: float = 1.008, energy_eV: float = 0.5, z0: float = 12.0,
                        temperature_K: float = 300.0, seed: int = SEED, traj_offset: int = 0):
    """IESH scattering workload: one hydrogen atom with three degrees of
    freedom approaching a metal along -z at energy_eV translational energy.
    The metal band has nstates - 1 evenly spaced levels on [-0.5, 0.5] Hartree
    with V_k = coupling sqrt(de) (TrapezoidalRule), Fermi level 0, electronic
    temperature 300 K, nelectrons electrons.  Impurity:
    U0 = kxy (x^2 + y^2)/2 + A exp(-a z), a repulsive wall with its turning
    point near z = 2 at 0.5 eV, and h = delta - B exp(-b z), an affinity level
    2.2 eV above the Fermi level far from the surface that crosses it at
    z = 2.2, so the atom charges up and excites electron-hole pairs at the
    turning point.  Initial p_z Gaussian around -sqrt(2 m E) (5 % spread),
    lateral momenta and positions thermal at 300 K, occupations Fermi-Dirac
    sampled by the engine.  dt = 0.1 fs; 1 ps is 10 000 steps."""
    M = nstates - 1
    eps, w = trapezoidal_rule(M, -0.5, 0.5)
    mass = mass_amu * AMU_AU
    T = temperature_K * KELVIN_AU
    omega_xy = 0.002
    kxy = mass * omega_xy**2
    params = dict(kxy=kxy, A=0.2, a=1.2, delta=0.08, B=0.3, b=0.6)
    rng = np.random.default_rng([seed, traj_offset, 5])
    p0 = np.sqrt(2.0 * mass * energy_eV * EV_AU)
    r0 = np.zeros((ntraj, 3))
    v0 = np.zeros((ntraj, 3))
    r0[:, 0:2] = rng.standard_normal((ntraj, 2)) * np.sqrt(T / kxy)
    r0[:, 2] = z0
    v0[:, 0:2] = rng.standard_normal((ntraj, 2)) * np.sqrt(T / mass)
    v0[:, 2] = -(p0 + 0.05 * p0 * rng.standard_normal(ntraj)) / mass
    return dict(eps=eps, V=coupling * np.sqrt(w), params=params, mass=mass, beta=1.0 / T, nstates=nstates,
                nelectrons=nelectrons, r0=r0, v0=v0, dt=0.1 * AU_PER_FS)


def newns_anderson_rpiesh(ntraj: int, nbeads: int, **kw):
    """Ring-polymer IESH workload: the IESH scattering workload's positions and
    velocities become the centroids, and the beads spread about them as a
    free ring polymer at the electronic temperature T: with
    beta_n = beta / nbeads and omega_n = nbeads / beta, the internal normal
    modes (eigenvectors of the cyclic bead Laplacian, eigenvalues
    4 sin^2(k pi / nbeads)) are Gaussian with variance
    1 / (beta_n m omega_n^2 4 sin^2(k pi / nbeads)), and the bead velocities
    are thermal at beta_n about the centroid velocity.  r0, v0:
    (ntraj, nbeads, 3), every centroid exactly the workload's value."""
    wl = newns_anderson_iesh(ntraj, **kw)
    B = nbeads
    m, beta = wl["mass"], wl["beta"]
    bn, wn = beta / B, B / beta
    rng = np.random.default_rng([kw.get("seed", SEED), kw.get("traj_offset", 0), 6])
    lap = 2.0 * np.eye(B) - np.roll(np.eye(B), 1, axis=1) - np.roll(np.eye(B), -1, axis=1)
    lam, E = np.linalg.eigh(lap)
    sd = np.zeros(B)
    internal = lam > 1e-9
    sd[internal] = 1.0 / np.sqrt(bn * m * wn * wn * lam[internal])
    q = rng.standard_normal((ntraj, 3, B)) * sd
    dr = np.einsum("bk,tdk->tbd", E, q)
    dv = rng.standard_normal((ntraj, B, 3)) / np.sqrt(bn * m)
    dr -= dr.mean(axis=1, keepdims=True)
    dv -= dv.mean(axis=1, keepdims=True)
    wl["r0"] = wl["r0"][:, None, :] + dr
    wl["v0"] = wl["v0"][:, None, :] + dv
    wl["nbeads"] = B
    return wl


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
