"""GPU parity of ring-polymer IESH (RingPolymerSimulation{AdiabaticIESH},
rpiesh.jl, integrated by BCBWavefunction, bcb_wavefunction.jl:37-69).

The oracle (iesh_oracle.run_rpiesh) takes dense LAPACK eigendecompositions
of every bead's and the centroid's Hamiltonian, the exact propagator and
explicit determinants; the engine uses secular roots, the Chebyshev
propagator and the determinant lemma, so the plain FP64 path agrees to
rounding: identical Fermi-Dirac occupations, hop sequences and
frustrated-hop counts, bead positions, velocities and orbitals to 1e-8.
"""
import numpy as np
import pytest

import iesh_oracle as IO
from nqcd_gb300 import _lib as L
from nqcd_gb300 import workload as WL
from test_gpu_iesh import compare_with_oracle, make_iesh, oracle_model, run_engine

pytestmark = pytest.mark.gpu


def run_pair(wl, n, nsteps, seed, **kw):
    fin = run_engine(wl, n, nsteps, seed, nbeads=wl["nbeads"], **kw)
    okw = dict(rescaling=kw.get("rescaling", 0))
    if kw.get("init") == L.INIT_GIVEN:
        okw["initial_state"] = kw["state0_arr"]
    o = IO.run_rpiesh(oracle_model(wl), mass=wl["mass"], ne=wl["nelectrons"], beta=wl["beta"], r0=wl["r0"],
                      v0=wl["v0"], dt=wl["dt"], nsteps=nsteps, seed=seed, **okw)
    return fin, o


@pytest.mark.parametrize("nstates,nelectrons,nbeads,n,nsteps,z0", [(20, 10, 4, 8, 400, 3.5), (80, 40, 4, 3, 300, 3.0),
                                                                    (24, 12, 8, 4, 300, 3.2), (16, 6, 32, 2, 200, 3.2)])
def test_rpiesh_fp64_matches_oracle(nstates, nelectrons, nbeads, n, nsteps, z0):
    wl = WL.newns_anderson_rpiesh(n, nbeads, nstates=nstates, nelectrons=nelectrons, z0=z0)
    fin, o = run_pair(wl, n, nsteps, 3)
    assert fin["stats"].unconverged_roots == 0
    assert fin["r"].shape == (n, nbeads, 3)
    compare_with_oracle(fin, o, n)
    if nstates == 80:
        assert sum(len(h) for h in o["hops"]) > 0  # the case exercises hops


def test_rpiesh_given_occupations_and_rescaling_modes():
    n, nsteps = 4, 300
    wl = WL.newns_anderson_rpiesh(n, 4, nstates=40, nelectrons=20, z0=3.0)
    occ0 = np.tile(np.arange(20, dtype=np.int32)[::-1], (n, 1)).copy()
    for rescaling in (1, 2):
        fin, o = run_pair(wl, n, nsteps, 5, rescaling=rescaling, init=L.INIT_GIVEN, state0_arr=occ0)
        compare_with_oracle(fin, o, n)


def test_rpiesh_energy_conserved_without_hops():
    # far from the surface no hop happens (300 steps of 0.1 fs at 0.5 eV take the atom from
    # z = 12 to about 6.5 bohr): the ring-polymer Hamiltonian is conserved by the symplectic
    # BCB integrator to O(dt^2)
    n, nsteps = 16, 300
    wl = WL.newns_anderson_rpiesh(n, 8, z0=12.0)
    fin = run_engine(wl, n, nsteps, 9, nbeads=8)
    assert np.all(fin["nhops"] == 0)
    drift = np.abs(fin["energy"][:, 1] - fin["energy"][:, 0])
    assert drift.max() < 1e-6 * np.abs(fin["energy"][:, 0]).max(), drift.max()


def test_rpiesh_fast_path_matches_plain():
    # FP32 electronic structure and propagation: bead positions and energies track the plain path
    # on the trajectories whose hop sequences agree
    n, nsteps, B = 64, 400, 8
    wl = WL.newns_anderson_rpiesh(n, B, z0=4.0)
    a = run_engine(wl, n, nsteps, 21, nbeads=B)
    b = run_engine(wl, n, nsteps, 21, nbeads=B, precision=L.PREC_FP32)
    same = [t for t in range(n) if np.array_equal(a["hop_log"][t], b["hop_log"][t])]
    assert len(same) > n // 2
    np.testing.assert_allclose(b["r"][same], a["r"][same], atol=2e-3, rtol=0)
    np.testing.assert_allclose(b["energy"][same], a["energy"][same], rtol=1e-5)
    for t in range(8):
        g = b["psi"][t].conj().T @ b["psi"][t]
        assert np.abs(g - np.eye(wl["nelectrons"])).max() < 2e-4


def test_rpiesh_shards_equal_the_single_ensemble():
    # random streams are keyed by the global trajectory index
    n, nsteps, B = 8, 200, 4
    wl = WL.newns_anderson_rpiesh(n, B, nstates=24, nelectrons=12, z0=3.2)
    full = run_engine(wl, n, nsteps, 17, nbeads=B)
    half = dict(wl, r0=wl["r0"][n // 2:], v0=wl["v0"][n // 2:])
    part = run_engine(half, n // 2, nsteps, 17, nbeads=B, traj_offset=n // 2)
    for key in ("r", "v", "psi", "state", "nhops", "energy"):
        np.testing.assert_array_equal(part[key], full[key][n // 2:], err_msg=key)


def test_rpiesh_run_dynamics_matches_engine():
    # RingPolymerSimulation[AdiabaticIESH] through run_dynamics, with per-trajectory arrays in
    # Julia's (ndofs, natoms, nbeads) shape, equals the engine fed the same beads
    import nqcd_gb300 as N

    n, B, nsteps = 4, 4, 150
    wl = WL.newns_anderson_rpiesh(n, B, nstates=20, nelectrons=10, z0=3.5)
    P = wl["params"]
    model = N.AndersonHolstein(N.AdsorbateMetal3D(P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"]),
                               N.TrapezoidalRule(19, -0.5, 0.5), coupling=0.04)
    np.testing.assert_allclose(model.V, wl["V"], rtol=1e-15)
    T = 1.0 / wl["beta"]
    sim = N.RingPolymerSimulation[N.AdiabaticIESH](N.Atoms(wl["mass"]), model, B, temperature=T)
    julia = lambda a: np.ascontiguousarray(a.transpose(0, 2, 1)[:, :, None, :])  # (n, 3, 1, B)
    dist = N.DynamicalDistribution(julia(wl["v0"]), julia(wl["r0"]), (3, 1, B)) * N.FermiDiracState(0.0, T)
    res = N.run_dynamics(sim, (0.0, nsteps * wl["dt"]), dist, output=(N.OutputFinal, N.OutputTotalEnergy),
                         trajectories=n, dt=wl["dt"], ensemble_algorithm=N.EnsembleGB300("fp64"), seed=7)
    eng = run_engine(wl, n, nsteps, 7, nbeads=B)
    fin = res["OutputFinal"]
    np.testing.assert_array_equal(fin["r"], eng["r"])
    np.testing.assert_array_equal(fin["v"], eng["v"])
    np.testing.assert_array_equal(fin["state"], eng["state"])
    np.testing.assert_allclose(res["OutputTotalEnergy"], eng["energy"].mean(axis=0), rtol=1e-14)


def test_rpiesh_time_series_matches_oracle():
    """Observables of ring-polymer IESH at save points (the reference's
    OutputKineticEnergy / OutputPotentialEnergy of a ring polymer: all beads,
    DynamicsUtils.jl:122-132 and rpiesh.jl:40-52; the centroid height; the
    impurity population of the centroid eigenstates), after each step's hops,
    against the oracle; the final energies include steps that ended with a hop."""
    n, nsteps, stride, B = 8, 300, 25, 4
    wl = WL.newns_anderson_rpiesh(n, B, nstates=20, nelectrons=10, z0=3.0)
    eng = make_iesh(wl, n, nbeads=B, save_stride=stride)
    try:
        eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
        obs = np.zeros((nsteps // stride + 1) * 4)
        _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], 5, observables=obs)
        fin = eng.get_final_iesh(wl["nstates"], wl["nelectrons"])
        fin["hop_log"] = eng.get_hop_log(eng.cfg.max_hops)
        fin["stats"] = st
    finally:
        eng.close()
    o = IO.run_rpiesh(oracle_model(wl), mass=wl["mass"], ne=wl["nelectrons"], beta=wl["beta"], r0=wl["r0"],
                      v0=wl["v0"], dt=wl["dt"], nsteps=nsteps, seed=5, save_stride=stride)
    compare_with_oracle(fin, o, n)
    print("hops:", sum(len(h) for h in o["hops"]))
    np.testing.assert_allclose(obs.reshape(-1, 4), o["obs"].mean(axis=1), rtol=1e-8, atol=1e-10)
