"""MDEF oracle -- TEST INFRASTRUCTURE ONLY.

A numpy FP64 restatement of NQCDynamics.jl's electronic-friction Langevin
dynamics on the Newns-Anderson (AndersonHolstein) model:

  MDEF_BAOAB.perform_step!   src/DynamicsMethods/IntegrationAlgorithms/mdef_baoab.jl:163-180
                             (one degree of freedom: run_mdef; the 3-D adsorbate with
                             the friction tensor's eigen-decomposition: run_mdef3d)
  step_O!                    src/DynamicsMethods/IntegrationAlgorithms/steps.jl:41-69
  DiabaticMDEF acceleration! src/DynamicsMethods/ClassicalMethods/mdef.jl:102-124
  friction!                  src/DynamicsMethods/ClassicalMethods/mdef.jl:131-140

The electronic structure is evaluated the way the reference's cache does it:
dense eigen-decomposition of the (1 + M) x (1 + M) one-electron Hamiltonian
(numpy.linalg.eigh, LAPACK), adiabatic derivative Z^T dH Z, Fermi-weighted
force, and the Gaussian-broadened friction
    Lambda = sum_nm -pi dH_nm dH_mn g_sigma(e_n - e_m) f'(e_n)
(the GaussianBroadening form of the reference's calculator package, which
is not vendored; its normalisation is restated here, parity unpinned).

Noise: one standard normal per degree of freedom and step from the engine's
Philox4x32-10 stream (key = seed, counter = (trajectory, step, NOISE stream,
0)), Box-Muller on the block's two 53-bit uniforms, restated in numpy, so the
oracle and the GPU integrate the same Wiener increments.

Model (restated from the AndersonHolstein definition: impurity level
h = U1 - U0, couplings V_k = V sqrt(w_k), bath levels e_k, state-independent
potential U0): a displaced-harmonic impurity
    U0(x) = k x^2 / 2,   U1(x) = k (x - g)^2 / 2 + Delta,   V constant,
and the bath of ShenviGaussLegendre(M, a, b) around the Fermi level mu.
"""
from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
RNG_NOISE = 3


def philox(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 (uint32 arrays)."""
    c0, c1, c2, c3 = (np.asarray(c, dtype=np.uint32) for c in (c0, c1, c2, c3))
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    mask = np.uint64(0xFFFFFFFF)
    for _ in range(10):
        p0 = c0.astype(np.uint64) * M0
        p1 = c2.astype(np.uint64) * M1
        hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
        lo0 = (p0 & mask).astype(np.uint32)
        hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
        lo1 = (p1 & mask).astype(np.uint32)
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = np.uint32((int(k0) + int(W0)) & 0xFFFFFFFF)
        k1 = np.uint32((int(k1) + int(W1)) & 0xFFFFFFFF)
    return c0, c1, c2, c3


def normal(seed: int, traj: np.ndarray, step: int, dof: int = 0) -> np.ndarray:
    """Standard normal per trajectory: Box-Muller on one Philox block,
    u1 = 1 - U53(w0, w1) in (0, 1], u2 = U53(w2, w3)."""
    traj = np.asarray(traj, dtype=np.uint64)
    w = philox((traj & np.uint64(0xFFFFFFFF)).astype(np.uint32), (traj >> np.uint64(32)).astype(np.uint32),
               np.full(traj.shape, step, np.uint32), np.full(traj.shape, RNG_NOISE + 16 * dof, np.uint32),
               seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    a = ((w[0].astype(np.uint64) << np.uint64(32)) | w[1].astype(np.uint64)) >> np.uint64(11)
    b = ((w[2].astype(np.uint64) << np.uint64(32)) | w[3].astype(np.uint64)) >> np.uint64(11)
    u1 = 1.0 - a.astype(np.float64) * 2.0**-53
    u2 = b.astype(np.float64) * 2.0**-53
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def shenvi_gauss_legendre(M: int, a: float, b: float, ef: float = 0.0):
    """Bath levels and weights (docs/src/NQCModels/systembathmodels.md:241-256):
    Gauss-Legendre halves below and above the Fermi level.  The upper half's
    shift is taken as (ef + b)/2, which maps the knots into [ef, b]."""
    x, w = np.polynomial.legendre.leggauss(M // 2)
    lo = 0.5 * (ef - a) * x + 0.5 * (a + ef)
    hi = 0.5 * (b - ef) * x + 0.5 * (ef + b)
    return np.concatenate([lo, hi]), np.concatenate([0.5 * (ef - a) * w, 0.5 * (b - ef) * w])


class NewnsAnderson:
    def __init__(self, *, k, g, delta, V, eps, weights, mu=0.0):
        self.k, self.g, self.delta, self.V, self.mu = k, g, delta, V, mu
        self.eps = np.asarray(eps, np.float64)
        self.Vk = V * np.sqrt(np.asarray(weights, np.float64))
        self.nstates = 1 + len(self.eps)

    def h(self, x):
        return self.k * self.g * (self.g / 2 - x) + self.delta

    def dh(self, x):
        return -self.k * self.g * np.ones_like(x)

    def dU0(self, x):
        return self.k * x

    def U0(self, x):
        return 0.5 * self.k * x * x

    def hamiltonian(self, x):
        n = len(x)
        N = self.nstates
        H = np.zeros((n, N, N))
        H[:, 0, 0] = self.h(x)
        H[:, 0, 1:] = self.Vk
        H[:, 1:, 0] = self.Vk
        idx = np.arange(1, N)
        H[:, idx, idx] = self.eps
        return H


def fermi(e, mu, beta):
    return 0.5 * (1.0 - np.tanh(0.5 * beta * (e - mu)))


def dfermi(e, mu, beta):
    f = fermi(e, mu, beta)
    return -beta * f * (1.0 - f)


def electronic(model, x, beta, sigma, want_friction=True):
    """Eigenvalues, Fermi-weighted force and broadened friction at x (vectorised)."""
    w, Z = np.linalg.eigh(model.hamiltonian(x))
    dh = model.dh(x)
    z0 = Z[:, 0, :]
    deps = dh[:, None] * z0 * z0  # (Z^T dH Z)_ii
    f = fermi(w, model.mu, beta)
    df = dfermi(w, model.mu, beta)
    F = model.dU0(x) + np.sum(deps * f + df * deps * w, axis=1)
    out = {"w": w, "F": F, "z0sq": z0 * z0}
    if want_friction:
        dH = dh[:, None, None] * z0[:, :, None] * z0[:, None, :]  # (Z^T dH Z)_nm
        de = w[:, :, None] - w[:, None, :]
        g = np.exp(-0.5 * de * de / sigma**2) / (sigma * np.sqrt(2 * np.pi))
        lam = np.sum(-np.pi * dH * dH * g * df[:, :, None], axis=(1, 2))
        out["friction"] = lam
    return out


def run_mdef(model: NewnsAnderson, *, mass, beta, sigma, x0, v0, dt, nsteps, seed, traj_offset=0,
             friction_fn=None, h_last=None, noise_dof=0):
    """BAOAB with friction in the tensor's eigenbasis (1 DoF: a scalar).
    friction_fn(x) may replace the exact friction (surrogate runs).
    h_last: length of the last step when the time span is not a whole number
    of steps; every sub-step of BAOAB reads the integrator's dt, the
    shortened one on the last step (mdef_baoab.jl:163-180, steps.jl:41-69),
    and the noise dW / sqrt(dt) is a standard normal whatever the step.
    noise_dof: the Philox stream of the degree of freedom (0 for the
    one-dimensional model)."""
    x = np.asarray(x0, np.float64).copy()
    v = np.asarray(v0, np.float64).copy()
    traj = np.arange(len(x), dtype=np.uint64) + np.uint64(traj_offset)
    T = 1.0 / beta
    half = 0.5
    k = -electronic(model, x, beta, sigma, want_friction=False)["F"] / mass
    for step in range(1, nsteps + 1):
        hs = h_last if (h_last is not None and step == nsteps) else dt  # this step's length
        v = v + (half * hs) * k                         # B
        x = x + (half * hs) * v                         # A
        if friction_fn is None:
            lam = electronic(model, x, beta, sigma)["friction"]
        else:
            lam = friction_fn(x)
        gam = np.maximum(lam / mass, 0.0)               # Lambda / (sqrt m sqrt m), clamp(gamma, 0, Inf)
        c1 = np.exp(-gam * hs)
        c2 = np.sqrt(1.0 - c1 * c1)
        noise = np.sqrt(T / mass) * normal(seed, traj, step, dof=noise_dof)
        v = c1 * v + c2 * noise                         # O
        x = x + (half * hs) * v                         # A
        k = -electronic(model, x, beta, sigma, want_friction=False)["F"] / mass
        v = v + (half * hs) * k                         # B
    return x, v


def electronic3d(model, r, mu, beta, sigma, want_friction=True):
    """The 3-D adsorbate (oracle.iesh_oracle.Metal3D, the IESH benchmark system)
    with DiabaticMDEF: eigen-decomposition of H(r), gradient
    dU0 + sum_i (d e_i f_i + f'_i d e_i e_i) with d_I e_i = (Z^T d_I H Z)_ii
    (mdef.jl:102-124), and the friction tensor
    Lambda_IJ = sum_nm -pi (Z^T d_I H Z)_nm (Z^T d_J H Z)_mn g_sigma(e_n - e_m) f'(e_n)
    over the three coordinates.  r: (n, 3)."""
    w, Z = np.linalg.eigh(model.hamiltonian(r))
    gh = model.grad_h(r)                                   # d_I h; d_I H = d_I h e_0 e_0^T
    z0 = Z[:, 0, :]
    dH = gh[:, :, None, None] * (z0[:, None, :, None] * z0[:, None, None, :])  # (n, 3, N, N)
    deps = np.einsum("tInn->tIn", dH)
    f = fermi(w, mu, beta)
    df = dfermi(w, mu, beta)
    F = model.grad_U0(r) + np.sum(deps * (f + df * w)[:, None, :], axis=2)
    out = {"w": w, "F": F}
    if want_friction:
        de = w[:, :, None] - w[:, None, :]
        g = np.exp(-0.5 * de * de / sigma**2) / (sigma * np.sqrt(2 * np.pi))
        out["friction"] = np.einsum("tInm,tJmn,tnm,tn->tIJ", dH, dH, -np.pi * g, df)
    return out


def run_mdef3d(model, *, mass, mu, beta, sigma, r0, v0, dt, nsteps, seed, traj_offset=0, h_last=None):
    """MDEF_BAOAB on the 3-D adsorbate: B, A, O with the friction tensor's
    eigen-decomposition (steps.jl:41-69: Lambda / m, eigenvalues clamped at 0,
    c1 = exp(-gamma dt), c2 = sqrt(1 - c1^2), v <- C c1 C^T v + C c2 C^T noise,
    one standard normal per degree of freedom I from the Philox stream of dof I),
    A, B.  r0, v0: (n, 3).  Returns r, v."""
    r = np.asarray(r0, np.float64).copy()
    v = np.asarray(v0, np.float64).copy()
    n = len(r)
    traj = np.arange(n, dtype=np.uint64) + np.uint64(traj_offset)
    T = 1.0 / beta
    k = -electronic3d(model, r, mu, beta, sigma, want_friction=False)["F"] / mass
    for step in range(1, nsteps + 1):
        hs = h_last if (h_last is not None and step == nsteps) else dt
        v = v + (0.5 * hs) * k                                         # B
        r = r + (0.5 * hs) * v                                         # A
        gam, C = np.linalg.eigh(electronic3d(model, r, mu, beta, sigma)["friction"] / mass)
        gam = np.maximum(gam, 0.0)
        c1 = np.exp(-gam * hs)
        c2 = np.sqrt(1.0 - c1 * c1)
        noise = np.sqrt(T / mass) * np.stack([normal(seed, traj, step, dof=I) for I in range(3)], axis=1)
        v = np.einsum("tij,tj->ti", C, c1 * np.einsum("tji,tj->ti", C, v)) + \
            np.einsum("tij,tj->ti", C, c2 * np.einsum("tji,tj->ti", C, noise))  # O
        r = r + (0.5 * hs) * v                                         # A
        k = -electronic3d(model, r, mu, beta, sigma, want_friction=False)["F"] / mass
        v = v + (0.5 * hs) * k                                         # B
    return r, v


def energy3d(model, r, v, mass, mu, beta):
    w, _ = np.linalg.eigh(model.hamiltonian(r))
    return 0.5 * mass * np.sum(v * v, axis=1) + model.U0(r) + np.sum(w * fermi(w, mu, beta), axis=1)


def energy(model, x, v, mass, beta):
    """Classical potential of DiabaticMDEF (mdef.jl:162-175) plus kinetic energy."""
    w, _ = np.linalg.eigh(model.hamiltonian(x))
    return 0.5 * mass * v * v + model.U0(x) + np.sum(w * fermi(w, model.mu, beta), axis=1)


def cayley_half(n: int, beta: float, dt: float) -> np.ndarray:
    """cayley_propagator(beads, dt; half=true) (ring_polymer.jl:71-82): the
    principal square root of each mode's full-step Cayley matrix C; det C = 1,
    so sqrt(C) = (C + I) / sqrt(tr C + 2).  Returns [n][2][2]."""
    import oracle as O

    C = O.cayley(n, beta, dt)
    tr = C[:, 0, 0] + C[:, 1, 1]
    return (C + np.eye(2)[None]) / np.sqrt(tr + 2.0)[:, None, None]


def run_rpmdef(model: NewnsAnderson, *, mass, beta, sigma, x0, v0, dt, nsteps, seed, traj_offset=0):
    """RingPolymerSimulation{DiabaticMDEF} with BCOCB (bcocb.jl:79-105):
    B (bead forces, rpmdef.jl:30-55), half Cayley step of the free ring
    polymer in normal modes, O in bead space with each bead's friction at the
    ring-polymer temperature n T (steps.jl:71-107, noise per bead from the
    Philox normal stream with dof = bead), half Cayley step, B.
    x0, v0: (ntraj, nbeads).  Returns x, v (ntraj, nbeads)."""
    import oracle as O

    x = np.asarray(x0, np.float64).copy()
    v = np.asarray(v0, np.float64).copy()
    n, B = x.shape
    traj = np.arange(n, dtype=np.uint64) + np.uint64(traj_offset)
    U = O.nm_transform(B)             # U[j, k]: bead j, mode k
    ch = cayley_half(B, beta, dt)     # omega_n = n / beta (RingPolymerParameters at the physical temperature)
    Trp = B / beta

    def force(x):
        return -electronic(model, x.ravel(), beta, sigma, want_friction=False)["F"].reshape(n, B) / mass

    def free_half(x, v):
        q, p = x @ U, v @ U           # to normal modes
        q2 = ch[:, 0, 0] * q + ch[:, 0, 1] * p
        p2 = ch[:, 1, 0] * q + ch[:, 1, 1] * p
        return q2 @ U.T, p2 @ U.T     # back to beads

    k = force(x)
    for step in range(1, nsteps + 1):
        v = v + (0.5 * dt) * k                                       # B
        x, v = free_half(x, v)                                       # C
        lam = electronic(model, x.ravel(), beta, sigma)["friction"].reshape(n, B)
        gam = np.maximum(lam / mass, 0.0)
        c1 = np.exp(-gam * dt)
        c2 = np.sqrt(1.0 - c1 * c1)
        xi = np.stack([normal(seed, traj, step, dof=j) for j in range(B)], axis=1)
        v = c1 * v + c2 * (np.sqrt(Trp / mass) * xi)                 # O
        x, v = free_half(x, v)                                       # C
        k = force(x)
        v = v + (0.5 * dt) * k                                       # B
    return x, v
