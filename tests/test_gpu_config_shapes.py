"""Plain FP64 GPU path against the oracle at the benchmark configurations'
own shapes, 1000 steps each (fixtures from tests/golden/make_config_shapes.py):

  MDEF, 200 band states, 256 trajectories: positions and velocities to 1e-8;
  ring-polymer MDEF, 200 band states, 4 beads, 32 trajectories: bead
      positions and velocities to 1e-8;
  IESH, 80 states and 40 electrons, 64 trajectories through the level
      crossing: identical Fermi-Dirac occupations, hop sequences and
      frustrated-hop counts; positions, velocities and orbitals to 1e-8.

These are the shapes where the secular solver's warm starts and the
Chebyshev cut-offs are stressed; the oracle diagonalises the dense matrices
(LAPACK) as the reference does.
"""
from pathlib import Path

import numpy as np
import pytest

from nqcd_gb300 import _lib as L
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _mdef_engine(wl, n, nbeads=0):
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_MDEF, L.MODEL_NEWNS_ANDERSON, L.PREC_FP64
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, 1, 1 + len(wl["eps"])
    params = np.array([wl["k"], wl["g"], wl["delta"], wl["mu"], wl["sigma"]])
    masses = np.array([wl["mass"]])
    eps = np.ascontiguousarray(wl["eps"])
    V = np.ascontiguousarray(wl["V"])
    cfg.nparams, cfg.params, cfg.masses = 5, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(eps), L.dptr(eps), L.dptr(V)
    cfg.beta = wl["beta"]
    cfg.ntraj_max = n
    cfg.nbeads_max = nbeads
    return L.Engine(cfg, [params, masses, eps, V])


def test_mdef_fp64_at_the_configuration_shape():
    g = np.load(GOLDEN / "mdef_c4.npz")
    n, M, nsteps, seed = len(g["x0"]), int(g["M"]), int(g["nsteps"]), int(g["seed"])
    wl = WL.newns_anderson_mdef(n, M=M)
    eng = _mdef_engine(wl, n)
    try:
        eng.set_initial(g["x0"].reshape(n, 1).copy(), g["v0"].reshape(n, 1).copy())
        _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], seed)
        fin = eng.get_final(1)
    finally:
        eng.close()
    assert st.unconverged_roots == 0
    np.testing.assert_allclose(fin["r"][:, 0], g["x"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(fin["v"][:, 0], g["v"], rtol=1e-8, atol=1e-12)


def test_rpmdef_fp64_at_the_configuration_shape():
    g = np.load(GOLDEN / "rpmdef_c4.npz")
    (n, B), M, nsteps, seed = g["x0"].shape, int(g["M"]), int(g["nsteps"]), int(g["seed"])
    wl = WL.newns_anderson_mdef(n, M=M)
    eng = _mdef_engine(wl, n, nbeads=B)
    try:
        eng.set_initial(np.ascontiguousarray(g["x0"]), np.ascontiguousarray(g["v0"]))
        _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], seed)
        fin = eng.get_final(B)
    finally:
        eng.close()
    assert st.unconverged_roots == 0
    np.testing.assert_allclose(fin["r"], g["x"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(fin["v"], g["v"], rtol=1e-8, atol=1e-12)


def test_iesh_fp64_at_the_configuration_shape():
    g = np.load(GOLDEN / "iesh_c5.npz")
    n, ne = g["state"].shape
    nsteps, seed = int(g["nsteps"]), int(g["seed"])
    wl = WL.newns_anderson_iesh(n, nstates=g["density"].shape[1], nelectrons=ne, z0=float(g["z0"]))
    P = wl["params"]
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_IESH, L.MODEL_NEWNS_ANDERSON_3D, L.PREC_FP64
    cfg.ndofs, cfg.natoms, cfg.nstates, cfg.nelectrons = 3, 1, wl["nstates"], ne
    params = np.array([P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"]])
    masses = np.array([wl["mass"]])
    eps = np.ascontiguousarray(wl["eps"])
    V = np.ascontiguousarray(wl["V"])
    cfg.nparams, cfg.params, cfg.masses = 6, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(eps), L.dptr(eps), L.dptr(V)
    cfg.beta = wl["beta"]
    cfg.ntraj_max = n
    cfg.init_kind = L.INIT_FERMI_DIRAC
    cfg.max_hops = g["hop_log"].shape[1]
    eng = L.Engine(cfg, [params, masses, eps, V])
    try:
        eng.set_initial(np.ascontiguousarray(g["r0"]), np.ascontiguousarray(g["v0"]))
        _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], seed)
        fin = eng.get_final_iesh(wl["nstates"], ne)
        log = eng.get_hop_log(cfg.max_hops)
    finally:
        eng.close()
    assert st.unconverged_roots == 0
    nh = int((g["hop_log"][:, :, 0] >= 0).sum())
    assert nh >= n // 4, nh  # the case exercises hops
    for t in range(n):
        got = [tuple(x) for x in log[t] if x[0] >= 0]
        want = [tuple(x) for x in g["hop_log"][t] if x[0] >= 0]
        assert got == want, (t, got, want)
        assert fin["nhops"][t] == len(want), t
    np.testing.assert_array_equal(fin["nfrustrated"], g["nfrustrated"])
    np.testing.assert_array_equal(fin["state"], g["state"])
    np.testing.assert_allclose(fin["r"], g["r"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(fin["v"], g["v"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(fin["energy"], g["energy"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(np.sum(np.abs(fin["psi"]) ** 2, axis=2), g["density"], atol=1e-8)
    k = g["psi_re"].shape[0]
    np.testing.assert_allclose(fin["psi"][:k], g["psi_re"] + 1j * g["psi_im"], atol=1e-8)
