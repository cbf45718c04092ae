"""GPU parity of the IESH kernel (independent-electron surface hopping on the
three-dimensional Newns-Anderson adsorbate).

The oracle follows the reference's algorithm with dense LAPACK
eigendecompositions, the exact propagator U exp(-i mu dt) U^H and explicit
determinants for every hop candidate; the engine uses the secular roots of
the arrowhead Hamiltonian, a Chebyshev propagator converged to 1e-17 and the
determinant lemma.  Agreement is to rounding, not bitwise:
  plain FP64 path: identical Fermi-Dirac occupations, hop sequences and
      frustrated-hop counts; positions, velocities and orbitals to 1e-8;
  fast FP32 path: ensemble observables within their sampling error.
The estimate screen of the reference (iesh.jl:251-254) never changes a
result: runs with and without it are bitwise equal.
"""
import numpy as np
import pytest

import iesh_oracle as IO
from nqcd_gb300 import _lib as L
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def make_iesh(wl, ntraj, precision=L.PREC_FP64, rescaling=0, init=L.INIT_FERMI_DIRAC, max_hops=32, save_stride=0,
              exact=0, method=L.METHOD_IESH, decoherence=0.0, nbeads=0, traj_offset=0, gap_fp64=0.0):
    P = wl["params"]
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision, cfg.rescaling = method, L.MODEL_NEWNS_ANDERSON_3D, precision, rescaling
    cfg.ndofs, cfg.natoms, cfg.nstates, cfg.nelectrons = 3, 1, wl["nstates"], wl["nelectrons"]
    params = np.array([P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"]])
    masses = np.array([wl["mass"]])
    eps = np.ascontiguousarray(wl["eps"])
    V = np.ascontiguousarray(wl["V"])
    cfg.nparams, cfg.params, cfg.masses = 6, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(eps), L.dptr(eps), L.dptr(V)
    cfg.beta = wl["beta"]
    cfg.ntraj_max = ntraj
    cfg.init_kind = init
    cfg.max_hops = max_hops
    cfg.save_stride = save_stride
    cfg.exact_hop_probability = exact
    cfg.decoherence_C = decoherence
    cfg.nbeads_max = nbeads  # > 1: RingPolymerSimulation{AdiabaticIESH}
    cfg.traj_offset = traj_offset
    cfg.gap_fp64 = gap_fp64
    return L.Engine(cfg, [params, masses, eps, V])


def oracle_model(wl):
    P = wl["params"]
    return IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                      V=wl["V"])


def run_engine(wl, n, nsteps, seed, state0_arr=None, mapping=None, **kw):
    eng = make_iesh(wl, n, **kw)
    try:
        if mapping:
            eng.set_mapping(mapping)
        eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]), state0=state0_arr)
        _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], seed)
        fin = eng.get_final_iesh(wl["nstates"], wl["nelectrons"])
        fin["hop_log"] = eng.get_hop_log(eng.cfg.max_hops)
        fin["stats"] = st
        return fin
    finally:
        eng.close()


def compare_with_oracle(fin, o, n):
    for t in range(n):
        log = [tuple(x) for x in fin["hop_log"][t] if x[0] >= 0]
        assert log == [tuple(h) for h in o["hops"][t]], (t, log, o["hops"][t])
    np.testing.assert_array_equal(fin["nfrustrated"], o["nfrustrated"])
    np.testing.assert_array_equal(fin["state"], o["state"])
    np.testing.assert_allclose(fin["r"], o["r"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(fin["v"], o["v"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(fin["psi"], o["psi"], atol=1e-8)
    np.testing.assert_allclose(fin["energy"], o["energy"], rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("nstates,nelectrons,n,nsteps,z0", [(20, 10, 12, 500, 3.5), (80, 40, 4, 300, 3.0)])
def test_iesh_fp64_matches_oracle(nstates, nelectrons, n, nsteps, z0):
    wl = WL.newns_anderson_iesh(n, nstates=nstates, nelectrons=nelectrons, z0=z0)
    fin = run_engine(wl, n, nsteps, 3)
    assert fin["stats"].unconverged_roots == 0
    o = IO.run_iesh(oracle_model(wl), mass=wl["mass"], ne=nelectrons, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"],
                    dt=wl["dt"], nsteps=nsteps, seed=3)
    compare_with_oracle(fin, o, n)
    if nstates == 80:
        assert sum(len(h) for h in o["hops"]) > 0  # the case exercises hops


def test_iesh_given_occupations_and_rescaling_modes():
    n, nsteps = 4, 300
    wl = WL.newns_anderson_iesh(n, nstates=40, nelectrons=20, z0=3.0)
    occ0 = np.tile(np.arange(20, dtype=np.int32)[::-1], (n, 1)).copy()  # ground state, reversed electron order
    for rescaling in (1, 2):
        fin = run_engine(wl, n, nsteps, 5, rescaling=rescaling, init=L.INIT_GIVEN, state0_arr=occ0)
        o = IO.run_iesh(oracle_model(wl), mass=wl["mass"], ne=20, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"],
                        dt=wl["dt"], nsteps=nsteps, seed=5, rescaling=rescaling, initial_state=occ0)
        compare_with_oracle(fin, o, n)


@pytest.mark.parametrize("precision", [L.PREC_FP64, L.PREC_FP32])
def test_iesh_estimate_screen_never_changes_results(precision):
    n, nsteps = 16, 400
    wl = WL.newns_anderson_iesh(n, z0=3.5)
    a = run_engine(wl, n, nsteps, 7, precision=precision)
    b = run_engine(wl, n, nsteps, 7, precision=precision, exact=1)
    for key in ("r", "v", "psi", "state", "nhops", "nfrustrated", "hop_log", "energy"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
    assert b["stats"].hop_evaluations == n * nsteps
    assert a["stats"].hop_evaluations < b["stats"].hop_evaluations


@pytest.mark.parametrize("cores,nbeads,z0", [(0, 0, 3.0), (1, 0, 3.0), (0, 4, 3.0), (0, 0, None)])
def test_iesh_gram_bound_never_changes_results(cores, nbeads, z0):
    """FP32 path: the hop tests whose estimate the Gram-matrix bound settles skip the LU of the
    overlap matrix; every result equals that of the LU in every step (iesh_lu_always = 1).  Through
    the level crossing (z0 = 3) the orbitals leave the occupied space and many steps still need the
    LU; on the benchmark's scattering workload almost none do."""
    n, nsteps = 64, 600
    kz = {} if z0 is None else dict(z0=z0)
    wl = WL.newns_anderson_rpiesh(n, nbeads, **kz) if nbeads else WL.newns_anderson_iesh(n, **kz)
    kw = dict(precision=L.PREC_FP32, nbeads=nbeads)
    a = run_engine(wl, n, nsteps, 17, mapping=dict(iesh_cores=cores), **kw)
    b = run_engine(wl, n, nsteps, 17, mapping=dict(iesh_cores=cores, iesh_lu_always=1), **kw)
    if z0 is not None:
        assert b["stats"].hops > 0
    for key in ("r", "v", "psi", "state", "nhops", "nfrustrated", "hop_log", "energy"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
    assert a["stats"].hop_evaluations == b["stats"].hop_evaluations
    assert b["stats"].overlap_factorizations == n * nsteps
    print("overlap LUs with the bound:", a["stats"].overlap_factorizations, "of", n * nsteps, "z0", z0)
    assert a["stats"].hop_evaluations <= a["stats"].overlap_factorizations < n * nsteps
    if z0 is None:
        assert a["stats"].overlap_factorizations < n * nsteps // 2


def test_iesh_fp64_factorizes_every_step():
    n, nsteps = 8, 100
    wl = WL.newns_anderson_iesh(n, z0=3.0)
    fin = run_engine(wl, n, nsteps, 17)
    assert fin["stats"].overlap_factorizations == n * nsteps


@pytest.mark.parametrize("precision,tol", [(L.PREC_FP64, 1e-10), (L.PREC_FP32, 2e-4)])
def test_iesh_orbitals_stay_orthonormal(precision, tol):
    n, nsteps = 8, 1000
    wl = WL.newns_anderson_iesh(n, z0=4.0)
    fin = run_engine(wl, n, nsteps, 11, precision=precision)
    for t in range(n):
        g = fin["psi"][t].conj().T @ fin["psi"][t]
        assert np.abs(g - np.eye(wl["nelectrons"])).max() < tol


def test_iesh_fast_path_observables():
    n, nsteps, stride = 1024, 1500, 100
    wl = WL.newns_anderson_iesh(n, z0=5.0)
    res = {}
    for prec in (L.PREC_FP64, L.PREC_FP32):
        eng = make_iesh(wl, n, precision=prec, save_stride=stride)
        try:
            eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
            obs = np.zeros((nsteps // stride + 1) * 4)
            out, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], 13, observables=obs)
            fin = eng.get_final_iesh(wl["nstates"], wl["nelectrons"])
            res[prec] = (obs.reshape(-1, 4), fin, st)
        finally:
            eng.close()
    (oa, fa, sa), (ob, fb, sb) = res[L.PREC_FP64], res[L.PREC_FP32]
    assert sa.hops > 0
    # same Fermi-Dirac start (FP64 roots on both paths)
    np.testing.assert_allclose(ob[0], oa[0], rtol=1e-5, atol=1e-6)
    # ensemble means along the run: height, kinetic energy, impurity population
    np.testing.assert_allclose(ob[:, 0], oa[:, 0], rtol=0.01)
    np.testing.assert_allclose(ob[:, 1], oa[:, 1], rtol=0.01)
    se = fa["nhops"].std() / np.sqrt(n)
    assert abs(fb["nhops"].mean() - fa["nhops"].mean()) <= 3 * se + 0.01
    assert np.mean(fa["nhops"] == fb["nhops"]) > 0.9


def test_iesh_decoherence_edc_fp64_matches_oracle():
    """IESH with DecoherenceCorrectionEDC(0.1) (decoherence_corrections.jl:21-39,
    applied after every step, iesh.jl:424-441): hop sequences identical to the
    oracle's, r, v and orbitals to 1e-8, and the correction changes the run."""
    n, nsteps = 16, 600
    wl = WL.newns_anderson_iesh(n, nstates=20, nelectrons=10, z0=3.0)
    fin = run_engine(wl, n, nsteps, 11, decoherence=0.1)
    o = IO.run_iesh(oracle_model(wl), mass=wl["mass"], ne=10, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"],
                    dt=wl["dt"], nsteps=nsteps, seed=11, decoherence_C=0.1)
    compare_with_oracle(fin, o, n)
    plain = run_engine(wl, n, nsteps, 11)
    assert np.max(np.abs(plain["psi"] - fin["psi"])) > 1e-3
    norms = np.linalg.norm(fin["psi"], axis=1)
    np.testing.assert_allclose(norms, 1.0, atol=1e-10)


def test_iesh_fp32_near_degeneracy_fallback():
    """The FP32 path's FP64 near-degeneracy fallback: two bath levels 1e-6
    apart put adjacent roots closer than gap_fp64 = 1e-3 on a good part of the
    steps (how close the roots next to the pair come depends on the adsorbate
    level); those roots are solved again in FP64 and the couplings between
    them formed from the FP64 roots.  The refined steps are counted in every
    trajectory (nqcd_get_status, summed in nqcd_stats.electronics_fp64_steps),
    nothing is counted with the fallback off or on the plain path, and the FP32
    run stays within FP32 tolerance of the plain FP64 path."""
    n, nsteps = 64, 200
    wl = WL.newns_anderson_iesh(n, nstates=40, nelectrons=20, z0=3.0)
    eps = wl["eps"].copy()
    k = len(eps) // 2
    eps[k] = eps[k - 1] + 1e-6
    wl["eps"] = eps
    res = {}
    for name, prec, gap in (("fp64", L.PREC_FP64, 1e-3), ("fp32", L.PREC_FP32, 1e-3), ("fp32_off", L.PREC_FP32, 0.0)):
        eng = make_iesh(wl, n, precision=prec, gap_fp64=gap)
        try:
            eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
            _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], 21)
            fin = eng.get_final_iesh(wl["nstates"], wl["nelectrons"])
            fin["hop_log"] = eng.get_hop_log(eng.cfg.max_hops)
            res[name] = (fin, st, eng.get_status()["fp64_steps"])
        finally:
            eng.close()
    (f64, s64, c64), (f32, s32, c32), (foff, soff, coff) = res["fp64"], res["fp32"], res["fp32_off"]
    assert np.all(c32 > 0) and np.all(c32 <= nsteps) and s32.electronics_fp64_steps == int(c32.sum())
    assert np.all(c64 == 0) and np.all(coff == 0) and soff.electronics_fp64_steps == 0
    print("max |psi - psi_fp64|: fallback", np.abs(f32["psi"] - f64["psi"]).max(), "off",
          np.abs(foff["psi"] - f64["psi"]).max())
    # trajectories whose hop sequences agree (the FP32 path may flip a near-tie hop)
    same = np.array([np.array_equal(a[a[:, 0] >= 0], b[b[:, 0] >= 0]) for a, b in zip(f32["hop_log"], f64["hop_log"])])
    assert same.mean() > 0.9
    np.testing.assert_allclose(f32["r"][same], f64["r"][same], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(f32["v"][same], f64["v"][same], rtol=1e-3, atol=1e-7)
    np.testing.assert_allclose(f32["energy"][:, 1].mean(), f64["energy"][:, 1].mean(), rtol=1e-4)


def test_iesh_fp64_shortened_last_step_matches_oracle():
    """A time span that is not a whole number of steps: Verlet and the
    propagator take the shortened last step (integrator.dt,
    verlet_with_electronics.jl:42-69), the hop probability keeps the proposed
    full dt (iesh.jl:390-398); identical hop sequences, r, v and orbitals to
    1e-8 of the oracle."""
    n, whole = 8, 300
    wl = WL.newns_anderson_iesh(n, nstates=20, nelectrons=10, z0=3.0)
    t1 = (whole + 0.6) * wl["dt"]
    eng = make_iesh(wl, n)
    try:
        eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
        _, st = eng.run(0.0, t1, wl["dt"], 3)
        fin = eng.get_final_iesh(wl["nstates"], wl["nelectrons"])
        fin["hop_log"] = eng.get_hop_log(eng.cfg.max_hops)
    finally:
        eng.close()
    assert st.traj_steps == n * (whole + 1)
    o = IO.run_iesh(oracle_model(wl), mass=wl["mass"], ne=10, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"],
                    dt=wl["dt"], nsteps=whole + 1, seed=3, h_last=t1 - whole * wl["dt"])
    compare_with_oracle(fin, o, n)


def test_iesh_get_final_needs_the_orbital_form():
    """The final state of an IESH handle is the orbitals: the two-state
    get_final refuses it (the C call would write 40 x 80 orbitals per
    trajectory into 2 x 2 density-matrix buffers)."""
    wl = WL.newns_anderson_iesh(4, nstates=16, nelectrons=8)
    eng = make_iesh(wl, 4)
    try:
        eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
        eng.run(0.0, 2 * wl["dt"], wl["dt"], 1)
        with pytest.raises(ValueError, match="get_final_iesh"):
            eng.get_final(3)
        fin = eng.get_final_iesh(wl["nstates"], wl["nelectrons"])
        assert fin["psi"].shape == (4, 16, 8)
    finally:
        eng.close()
