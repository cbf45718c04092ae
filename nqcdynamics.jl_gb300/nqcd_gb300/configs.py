"""Engines for the benchmark configurations (C1-C5 of the reference's
headline benchmark), built from the synthetic workloads in workload.py.

C1  FSSH, Tully single avoided crossing, 10 000 trajectories
C2  FSSH, Ohmic spin-boson (100 modes), 100 000 trajectories   (bench.py default)
C3  RPSH, Tully 1-3 mixed, bead counts {4, 8, 16, 32}, 200 000 trajectories
C4  MDEF, Newns-Anderson, 200 band states, 50 000 trajectories
C5  IESH, Newns-Anderson, 40 electrons in 80 states, 20 000 trajectories
"""
from __future__ import annotations

import numpy as np

from . import workload as WL

TULLY_PARAMS = {1: (0.01, 1.6, 0.005, 1.0), 2: (0.1, 0.28, 0.015, 0.06, 0.05), 3: (6e-4, 0.1, 0.9)}


def tully_fssh(L, ntraj, precision, model=1, mass=2000.0, rescaling=0, max_hops=0, traj_offset=0):
    """C1: FSSH on a Tully model, one degree of freedom, adiabatic state 1."""
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision, cfg.rescaling = L.METHOD_FSSH, model, precision, rescaling
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, 1, 2
    p = np.asarray(TULLY_PARAMS[model], np.float64)
    m = np.array([mass])
    cfg.nparams, cfg.params, cfg.masses = len(p), L.dptr(p), L.dptr(m)
    cfg.ntraj_max = ntraj
    cfg.init_kind, cfg.init_state = L.INIT_ADIABATIC_PURE, 0
    cfg.max_hops = max_hops
    cfg.gap_fp64 = 1e-3
    cfg.traj_offset = traj_offset
    return L.Engine(cfg, [p, m])


def spinboson_fssh(L, w, c, ntraj, nmodes, precision, save_stride=0, traj_offset=0, method=None):
    """C2: FSSH (or Ehrenfest) on the Ohmic spin-boson model, unit masses,
    diabatic pure state 1 (frequencies w, couplings c)."""
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = method or L.METHOD_FSSH, L.MODEL_SPINBOSON, precision
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, nmodes, 2
    params = np.array([0.0, 1.0])
    masses = np.ones(nmodes)
    c = np.ascontiguousarray(c, np.float64)
    w = np.ascontiguousarray(w, np.float64)
    cfg.nparams, cfg.params, cfg.masses = 2, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = nmodes, L.dptr(c), L.dptr(w)
    cfg.ntraj_max = ntraj
    cfg.init_kind, cfg.init_state = L.INIT_DIABATIC_PURE, 0
    cfg.save_stride = save_stride
    cfg.gap_fp64 = 1e-3
    cfg.traj_offset = traj_offset
    return L.Engine(cfg, [params, masses, c, w])


def tully_inputs(ntraj, x0=-10.0, p0=10.0, mass=2000.0):
    return np.full((ntraj, 1), x0), np.full((ntraj, 1), p0 / mass)


def rpsh_tully(L, ntraj, precision, bmax=32, beta=1024.0, mass=2000.0, terminate_x=10.0, rescaling=0, max_hops=0,
               traj_offset=0):
    """C3: ring-polymer surface hopping on Tully models (the handle's model is
    Tully 1; per-trajectory models come from nqcd_set_trajectory_models)."""
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision, cfg.rescaling = L.METHOD_RPSH, 1, precision, rescaling
    cfg.ndofs, cfg.natoms, cfg.nstates, cfg.nbeads_max = 1, 1, 2, bmax
    p = np.asarray(TULLY_PARAMS[1], np.float64)
    m = np.array([mass])
    cfg.nparams, cfg.params, cfg.masses = len(p), L.dptr(p), L.dptr(m)
    cfg.beta = beta
    cfg.ntraj_max = ntraj
    cfg.init_kind, cfg.init_state = L.INIT_ADIABATIC_PURE, 0
    cfg.max_hops = max_hops
    cfg.terminate_x = terminate_x
    cfg.gap_fp64 = 1e-3
    cfg.traj_offset = traj_offset
    return L.Engine(cfg, [p, m])


def rpsh_inputs(ntraj, bmax=32, mass=2000.0, x0=-9.5, seed=WL.SEED, traj_offset=0):
    """Models 1-3 round robin, bead counts uniform in {4, 8, 16, 32}, p0
    uniform in [8, 30], all beads at the centroid x0."""
    rng = np.random.default_rng([seed, traj_offset, 3])
    nb = rng.choice(np.array([4, 8, 16, 32], np.int32), ntraj).astype(np.int32)
    p0 = rng.uniform(8.0, 30.0, ntraj)
    r0 = np.full((ntraj, bmax), x0)
    v0 = np.repeat((p0 / mass)[:, None], bmax, axis=1)
    models = (1 + (np.arange(ntraj) + traj_offset) % 3).astype(np.int32)
    return r0, v0, nb, models


def mdef_newns_anderson(L, wl, ntraj, precision, surrogate=False, exact_friction_every=0, save_stride=0, traj_offset=0,
                        nbeads=0):
    """C4: MDEF (electronic-friction Langevin) on the Newns-Anderson model
    (nbeads > 1: ring-polymer MDEF with that many beads)."""
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_MDEF, L.MODEL_NEWNS_ANDERSON, precision
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, 1, 1 + len(wl["eps"])
    params = np.array([wl["k"], wl["g"], wl["delta"], wl["mu"], wl["sigma"]])
    masses = np.array([wl["mass"]])
    eps = np.ascontiguousarray(wl["eps"])
    V = np.ascontiguousarray(wl["V"])
    cfg.nparams, cfg.params, cfg.masses = 5, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(eps), L.dptr(eps), L.dptr(V)
    cfg.beta = wl["beta"]
    cfg.ntraj_max = ntraj
    cfg.save_stride = save_stride
    cfg.use_friction_surrogate = int(surrogate)
    cfg.exact_friction_every = exact_friction_every
    cfg.traj_offset = traj_offset
    cfg.nbeads_max = nbeads
    return L.Engine(cfg, [params, masses, eps, V])


def mdef_adsorbate3d(L, wl, ntraj, precision, save_stride=0, traj_offset=0, mu=0.0, sigma=0.01):
    """MDEF on the three-dimensional adsorbate of the IESH system (one atom,
    x, y, z): the friction tensor has its one nonzero eigenvalue along z."""
    P = wl["params"]
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_MDEF, L.MODEL_NEWNS_ANDERSON_3D, precision
    cfg.ndofs, cfg.natoms, cfg.nstates = 3, 1, 1 + len(wl["eps"])
    params = np.array([P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"], mu, sigma])
    masses = np.array([wl["mass"]])
    eps = np.ascontiguousarray(wl["eps"])
    V = np.ascontiguousarray(wl["V"])
    cfg.nparams, cfg.params, cfg.masses = 8, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(eps), L.dptr(eps), L.dptr(V)
    cfg.beta = wl["beta"]
    cfg.ntraj_max = ntraj
    cfg.save_stride = save_stride
    cfg.traj_offset = traj_offset
    return L.Engine(cfg, [params, masses, eps, V])


def iesh_newns_anderson(L, wl, ntraj, precision, rescaling=0, save_stride=0, max_hops=0, exact=0, traj_offset=0,
                        method=None, nbeads=0, gap_fp64=1e-3):
    """C5: IESH on the three-dimensional Newns-Anderson adsorbate, Fermi-Dirac
    initial occupations (method=L.METHOD_EHRENFEST_NA: EhrenfestNA on the same
    system; nbeads > 1: RingPolymerSimulation{AdiabaticIESH} with that many
    beads).  The FP32 path refines adjacent roots closer than gap_fp64 in
    FP64 (the near-degeneracy fallback)."""
    P = wl["params"]
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision, cfg.rescaling = (method or L.METHOD_IESH), L.MODEL_NEWNS_ANDERSON_3D, \
        precision, rescaling
    cfg.ndofs, cfg.natoms, cfg.nstates, cfg.nelectrons = 3, 1, wl["nstates"], wl["nelectrons"]
    params = np.array([P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"]])
    masses = np.array([wl["mass"]])
    eps = np.ascontiguousarray(wl["eps"])
    V = np.ascontiguousarray(wl["V"])
    cfg.nparams, cfg.params, cfg.masses = 6, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(eps), L.dptr(eps), L.dptr(V)
    cfg.beta = wl["beta"]
    cfg.ntraj_max = ntraj
    cfg.init_kind = L.INIT_FERMI_DIRAC
    cfg.save_stride = save_stride
    cfg.max_hops = max_hops
    cfg.exact_hop_probability = exact
    cfg.traj_offset = traj_offset
    cfg.nbeads_max = nbeads
    cfg.gap_fp64 = gap_fp64
    return L.Engine(cfg, [params, masses, eps, V])
