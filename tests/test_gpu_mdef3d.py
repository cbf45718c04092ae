"""MDEF with three degrees of freedom: one atom (x, y, z) above the metal of
the IESH system, DiabaticMDEF with the friction tensor of all three
coordinates (the reference's O-step diagonalises it, steps.jl:41-69).  The
impurity level depends on z alone, so the tensor's one nonzero eigenvalue
lies along z; x and y move in the harmonic U0 without friction or noise.

The oracle (mdef_oracle.run_mdef3d) diagonalises the dense Hamiltonian and
the 3x3 tensor with LAPACK; the engine uses the secular roots and the
tensor's eigenvector in closed form.  Agreement is to rounding:
  FP64 path: force and friction to 1e-9, positions and velocities after 300
             steps to 1e-8, energies to 1e-10;
  FP32 path: force and friction to 2e-3, ensemble observables within 2 % of
             the FP64 path.
"""
import numpy as np
import pytest

import iesh_oracle as IO
import mdef_oracle as MO
import nqcd_gb300 as N
from nqcd_gb300 import _lib as L
from nqcd_gb300 import configs as C
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu
SIGMA = 0.01


def oracle_model(wl):
    P = wl["params"]
    return IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                      V=wl["V"])


def test_mdef3d_force_and_friction():
    wl = WL.newns_anderson_iesh(8, nstates=41, nelectrons=20)
    z = np.linspace(0.8, 6.0, 97)
    r = np.stack([np.zeros_like(z), np.zeros_like(z), z], axis=1)
    ref = MO.electronic3d(oracle_model(wl), r, 0.0, wl["beta"], SIGMA)
    for prec, rtol in ((L.PREC_FP64, 1e-9), (L.PREC_FP32, 2e-3)):
        eng = C.mdef_adsorbate3d(L, wl, 8, prec, sigma=SIGMA)
        try:
            F, G = eng.mdef_evaluate(z)
        finally:
            eng.close()
        np.testing.assert_allclose(F, ref["F"][:, 2], rtol=rtol, atol=rtol * np.abs(ref["F"][:, 2]).max())
        np.testing.assert_allclose(G, ref["friction"][:, 2, 2], rtol=rtol,
                                   atol=rtol * np.abs(ref["friction"][:, 2, 2]).max())
    assert ref["friction"][:, 2, 2].max() > 0


def run_engine(wl, n, nsteps, seed, precision, save_stride=0):
    eng = C.mdef_adsorbate3d(L, wl, n, precision, save_stride=save_stride, sigma=SIGMA)
    try:
        eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
        obs = np.zeros((nsteps // max(save_stride, 1) + 1) * 4)
        _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], seed, observables=obs if save_stride else None)
        fin = eng.get_final(3)
        fin["stats"] = st
        fin["obs"] = obs.reshape(-1, 4)
        return fin
    finally:
        eng.close()


def test_mdef3d_fp64_matches_oracle():
    n, nsteps = 16, 300
    wl = WL.newns_anderson_iesh(n, nstates=41, nelectrons=20, z0=2.5)
    fin = run_engine(wl, n, nsteps, 41, L.PREC_FP64)
    assert fin["stats"].unconverged_roots == 0
    model = oracle_model(wl)
    r, v = MO.run_mdef3d(model, mass=wl["mass"], mu=0.0, beta=wl["beta"], sigma=SIGMA, r0=wl["r0"], v0=wl["v0"],
                         dt=wl["dt"], nsteps=nsteps, seed=41)
    np.testing.assert_allclose(fin["r"], r, rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(fin["v"], v, rtol=1e-8, atol=1e-12)
    e0 = MO.energy3d(model, wl["r0"], wl["v0"], wl["mass"], 0.0, wl["beta"])
    e1 = MO.energy3d(model, r, v, wl["mass"], 0.0, wl["beta"])
    np.testing.assert_allclose(fin["energy"][:, 0], e0, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(fin["energy"][:, 1], e1, rtol=1e-10, atol=1e-12)
    # the friction and the noise acted: the energy is not conserved
    assert np.abs(e1 - e0).max() > 1e-6


def test_mdef3d_fp32_tracks_fp64():
    n, nsteps, stride = 512, 400, 50
    wl = WL.newns_anderson_iesh(n, z0=2.5)
    a = run_engine(wl, n, nsteps, 7, L.PREC_FP64, save_stride=stride)
    b = run_engine(wl, n, nsteps, 7, L.PREC_FP32, save_stride=stride)
    for col in (0, 2):  # <z>, <KE>
        np.testing.assert_allclose(b["obs"][:, col], a["obs"][:, col], rtol=0.02)
    np.testing.assert_allclose(b["energy"][:, 1].mean(), a["energy"][:, 1].mean(), rtol=0.02)


def test_mdef3d_run_dynamics_matches_engine():
    n, nsteps = 16, 100
    wl = WL.newns_anderson_iesh(n, z0=2.5)
    P = wl["params"]
    model = N.AndersonHolstein(N.AdsorbateMetal3D(P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"]),
                               N.TrapezoidalRule(79, -0.5, 0.5), coupling=0.04)
    np.testing.assert_allclose(model.V, wl["V"])
    sim = N.Simulation[N.DiabaticMDEF](N.Atoms(wl["mass"]), model, friction_method=N.GaussianBroadening(SIGMA),
                                       temperature=1.0 / wl["beta"])
    dist = N.DynamicalDistribution(wl["v0"], wl["r0"], (3, 1))
    res = N.run_dynamics(sim, (0.0, nsteps * wl["dt"]), dist, output=(N.OutputFinal, N.OutputPosition),
                         trajectories=n, dt=wl["dt"], saveat=10 * wl["dt"], ensemble_algorithm=N.EnsembleGB300("fp64"),
                         seed=4)
    fin = run_engine(wl, n, nsteps, 4, L.PREC_FP64, save_stride=10)
    np.testing.assert_array_equal(res["OutputFinal"]["r"], fin["r"])
    np.testing.assert_array_equal(res["OutputPosition"], fin["obs"][:, 0])


def test_mdef3d_limits():
    """The 3-D adsorbate runs classical nuclei with the exact friction."""
    wl = WL.newns_anderson_iesh(4, nstates=41, nelectrons=20)
    P = wl["params"]
    params = np.array([P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"], 0.0, SIGMA])
    masses = np.array([wl["mass"]])
    eps, V = np.ascontiguousarray(wl["eps"]), np.ascontiguousarray(wl["V"])
    for kw in (dict(use_friction_surrogate=1), dict(nbeads_max=4)):
        cfg = L.nqcd_config()
        cfg.method, cfg.model, cfg.precision = L.METHOD_MDEF, L.MODEL_NEWNS_ANDERSON_3D, L.PREC_FP32
        cfg.ndofs, cfg.natoms, cfg.nstates = 3, 1, 41
        cfg.nparams, cfg.params, cfg.masses = 8, L.dptr(params), L.dptr(masses)
        cfg.nbath, cfg.bath_a, cfg.bath_b = 40, L.dptr(eps), L.dptr(V)
        cfg.beta, cfg.ntraj_max = wl["beta"], 4
        for k, val in kw.items():
            setattr(cfg, k, val)
        with pytest.raises(L.EngineError) as e:
            L.Engine(cfg, [params, masses, eps, V])
        assert e.value.code == L.NQCD_ERR_UNSUPPORTED
