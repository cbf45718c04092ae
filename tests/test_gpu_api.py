"""run_dynamics through the host mirror (nqcd_gb300.api) on the metal-surface
methods equals the direct engine runs of the benchmark configurations."""
import numpy as np
import pytest

import nqcd_gb300 as N
from nqcd_gb300 import _lib as L
from nqcd_gb300 import configs as C
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def test_iesh_run_dynamics_matches_engine():
    n, nsteps = 16, 200
    wl = WL.newns_anderson_iesh(n, z0=4.0)
    P = wl["params"]
    model = N.AndersonHolstein(N.AdsorbateMetal3D(P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"]),
                               N.TrapezoidalRule(79, -0.5, 0.5), coupling=0.04)
    np.testing.assert_allclose(model.V, wl["V"])
    sim = N.Simulation[N.AdiabaticIESH](N.Atoms(wl["mass"]), model)
    dist = N.DynamicalDistribution(wl["v0"], wl["r0"], (3, 1)) * N.FermiDiracState(0.0, 1.0 / wl["beta"])
    res = N.run_dynamics(sim, (0.0, nsteps * wl["dt"]), dist, output=(N.OutputFinal, N.OutputKineticEnergy),
                         trajectories=n, dt=wl["dt"], saveat=50 * wl["dt"], ensemble_algorithm=N.EnsembleGB300("fp64"),
                         seed=9)
    eng = C.iesh_newns_anderson(L, wl, n, L.PREC_FP64, save_stride=50)
    try:
        eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
        obs = np.zeros((nsteps // 50 + 1) * 4)
        eng.run(0.0, nsteps * wl["dt"], wl["dt"], 9, observables=obs)
        fin = eng.get_final_iesh(80, 40)
    finally:
        eng.close()
    np.testing.assert_array_equal(res["OutputFinal"]["r"], fin["r"])
    np.testing.assert_array_equal(res["OutputFinal"]["state"], fin["state"])
    np.testing.assert_array_equal(res["OutputKineticEnergy"], obs.reshape(-1, 4)[:, 1])
    assert len(res["Time"]) == nsteps // 50 + 1


def test_mdef_run_dynamics_matches_engine():
    n, nsteps = 32, 100
    wl = WL.newns_anderson_mdef(n, M=40)
    model = N.AndersonHolstein(N.DisplacedHarmonic(wl["k"], wl["g"], wl["delta"]),
                               N.ShenviGaussLegendre(40, -0.5, 0.5), coupling=0.02)
    np.testing.assert_allclose(model.V, wl["V"])
    sim = N.Simulation[N.DiabaticMDEF](N.Atoms(wl["mass"]), model, friction_method=N.GaussianBroadening(wl["sigma"]),
                                       temperature=1.0 / wl["beta"])
    dist = N.DynamicalDistribution(wl["v0"].reshape(n, 1), wl["x0"].reshape(n, 1), (1, 1))
    res = N.run_dynamics(sim, (0.0, nsteps * wl["dt"]), dist, output=(N.OutputFinal, N.OutputPosition),
                         trajectories=n, dt=wl["dt"], saveat=10 * wl["dt"], ensemble_algorithm=N.EnsembleGB300("fp64"),
                         seed=4)
    eng = C.mdef_newns_anderson(L, wl, n, L.PREC_FP64, save_stride=10)
    try:
        eng.set_initial(wl["x0"].reshape(n, 1).copy(), wl["v0"].reshape(n, 1).copy())
        obs = np.zeros((nsteps // 10 + 1) * 4)
        eng.run(0.0, nsteps * wl["dt"], wl["dt"], 4, observables=obs)
        fin = eng.get_final(1)
    finally:
        eng.close()
    np.testing.assert_array_equal(res["OutputFinal"]["r"], fin["r"])
    np.testing.assert_array_equal(res["OutputPosition"], obs.reshape(-1, 4)[:, 0])


def test_file_reduction_writes_each_trajectory(tmp_path):
    """FileReduction (reductions.jl:57-91) through run_dynamics: one group per
    trajectory holding the same final state the device reduction averages."""
    ntraj, nm = 64, 8
    model = N.SpinBoson(N.OhmicSpectralDensity(2.5, 0.1), nm, 0.0, 1.0)
    sim = N.Simulation[N.FSSH](N.Atoms(np.ones(nm)), model)
    rng = np.random.default_rng(5)
    r0, v0 = rng.normal(size=(ntraj, 1, nm)), rng.normal(size=(ntraj, 1, nm))
    dist = N.DynamicalDistribution(v0, r0, (1, nm)) * N.PureState(1, N.Diabatic())
    kw = dict(trajectories=ntraj, dt=0.05, seed=8, ensemble_algorithm=N.EnsembleGB300("fp64"))
    msg = N.run_dynamics(sim, (0.0, 2.0), dist, output=(N.OutputTotalEnergy, N.OutputSurfaceHops, N.OutputPosition,
                                                        N.OutputVelocity),
                         reduction=N.FileReduction(str(tmp_path / "sb.h5")), **kw)
    assert msg == f"Output written to {tmp_path / 'sb.npz'}."
    ref = N.run_dynamics(sim, (0.0, 2.0), dist, output=N.OutputFinal, **kw)["OutputFinal"]
    f = np.load(tmp_path / "sb.npz")
    for i in range(ntraj):
        g = f"trajectory_{i + 1}/"
        np.testing.assert_array_equal(f[g + "Time"], [0.0, 2.0])
        np.testing.assert_array_equal(f[g + "OutputTotalEnergy"], ref["energy"][i])
        assert f[g + "OutputSurfaceHops"] == ref["nhops"][i]
        np.testing.assert_array_equal(f[g + "OutputPosition"][:, 0], r0[i].ravel())
        np.testing.assert_array_equal(f[g + "OutputPosition"][:, 1], ref["r"][i])
        np.testing.assert_array_equal(f[g + "OutputVelocity"][:, 1], ref["v"][i])


def test_file_reduction_iesh(tmp_path):
    n, nsteps = 8, 100
    wl = WL.newns_anderson_iesh(n, z0=4.0)
    P = wl["params"]
    model = N.AndersonHolstein(N.AdsorbateMetal3D(P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"]),
                               N.TrapezoidalRule(79, -0.5, 0.5), coupling=0.04)
    sim = N.Simulation[N.AdiabaticIESH](N.Atoms(wl["mass"]), model)
    dist = N.DynamicalDistribution(wl["v0"], wl["r0"], (3, 1)) * N.FermiDiracState(0.0, 1.0 / wl["beta"])
    kw = dict(trajectories=n, dt=wl["dt"], ensemble_algorithm=N.EnsembleGB300("fp64"), seed=9)
    N.run_dynamics(sim, (0.0, nsteps * wl["dt"]), dist, output=(N.OutputPosition, N.OutputTotalEnergy,
                                                                N.OutputSurfaceHops),
                   reduction=N.FileReduction(str(tmp_path / "iesh")), **kw)
    ref = N.run_dynamics(sim, (0.0, nsteps * wl["dt"]), dist, output=N.OutputFinal, **kw)["OutputFinal"]
    f = np.load(tmp_path / "iesh.npz")
    for i in range(n):
        g = f"trajectory_{i + 1}/"
        np.testing.assert_array_equal(f[g + "OutputPosition"][:, 1], ref["r"][i])
        np.testing.assert_array_equal(f[g + "OutputTotalEnergy"], ref["energy"][i])
        assert f[g + "OutputSurfaceHops"] == ref["nhops"][i]
