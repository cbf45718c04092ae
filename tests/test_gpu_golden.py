"""GPU kernels against the committed golden fixtures (tests/golden/*.npz):
plain FP64 FSSH and RPSH bit for bit, MDEF and IESH to 1e-8."""
from pathlib import Path

import numpy as np
import pytest

from nqcd_gb300 import _lib as L
from nqcd_gb300 import configs as C
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
SEED = 20261203


def test_fssh_tully1_golden():
    g = np.load(GOLDEN / "fssh_tully1.npz")
    n = g["r0"].shape[0]
    eng = C.tully_fssh(L, n, L.PREC_FP64, max_hops=16)
    try:
        eng.set_initial(np.ascontiguousarray(g["r0"]), np.ascontiguousarray(g["v0"]))
        eng.run(0.0, 1500.0, 1.0, SEED)
        fin = eng.get_final(1)
        log = eng.get_hop_log(16)
    finally:
        eng.close()
    np.testing.assert_array_equal(fin["r"], g["r"])
    np.testing.assert_array_equal(fin["v"], g["v"])
    np.testing.assert_array_equal(fin["sig_re"], g["sigma_re"])
    np.testing.assert_array_equal(fin["state"], g["state"])
    np.testing.assert_array_equal(log, g["hop_log"])


def test_fssh_spinboson_golden():
    g = np.load(GOLDEN / "fssh_spinboson.npz")
    n, modes = g["r0"].shape
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_FSSH, L.MODEL_SPINBOSON, L.PREC_FP64
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, modes, 2
    params, masses = np.array([0.0, 1.0]), np.ones(modes)
    c, w = np.ascontiguousarray(g["c"]), np.ascontiguousarray(g["w"])
    cfg.nparams, cfg.params, cfg.masses = 2, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = modes, L.dptr(c), L.dptr(w)
    cfg.ntraj_max = n
    cfg.init_kind, cfg.init_state, cfg.max_hops = L.INIT_DIABATIC_PURE, 0, 16
    eng = L.Engine(cfg, [params, masses, c, w])
    try:
        eng.set_initial(np.ascontiguousarray(g["r0"]), np.ascontiguousarray(g["v0"]))
        eng.run(0.0, 5.0, 0.05, SEED)
        fin = eng.get_final(modes)
        log = eng.get_hop_log(16)
    finally:
        eng.close()
    np.testing.assert_array_equal(fin["r"], g["r"])
    np.testing.assert_array_equal(fin["v"], g["v"])
    np.testing.assert_array_equal(fin["sig_re"], g["sigma_re"])
    np.testing.assert_array_equal(fin["state"], g["state"])
    np.testing.assert_array_equal(log, g["hop_log"])


def test_rpsh_golden():
    g = np.load(GOLDEN / "rpsh_mixed.npz")
    n, bmax = g["r0"].shape
    eng = C.rpsh_tully(L, n, L.PREC_FP64, bmax=bmax, max_hops=16)
    try:
        eng.set_initial(np.ascontiguousarray(g["r0"]), np.ascontiguousarray(g["v0"]),
                        nbeads=np.ascontiguousarray(g["nbeads"]))
        eng.run(0.0, 800.0, 1.0, SEED)
        fin = eng.get_final(bmax)
        log = eng.get_hop_log(16)
    finally:
        eng.close()
    nb = g["nbeads"]
    for t in range(n):
        np.testing.assert_array_equal(fin["r"][t, : nb[t]], g["r"][t, : nb[t]])
        np.testing.assert_array_equal(fin["v"][t, : nb[t]], g["v"][t, : nb[t]])
    np.testing.assert_array_equal(fin["state"], g["state"])
    np.testing.assert_array_equal(fin["nsteps"], g["nsteps"])
    np.testing.assert_array_equal(log, g["hop_log"])
    np.testing.assert_array_equal(fin["energy"], g["energy"])


def test_mdef_golden():
    g = np.load(GOLDEN / "mdef_small.npz")
    n = len(g["x0"])
    k, gg, delta, mu, sigma, mass, beta, dt = g["params"]
    wl = dict(eps=g["eps"], V=g["V"], k=k, g=gg, delta=delta, mu=mu, sigma=sigma, mass=mass, beta=beta)
    eng = C.mdef_newns_anderson(L, wl, n, L.PREC_FP64)
    try:
        eng.set_initial(g["x0"].reshape(n, 1).copy(), g["v0"].reshape(n, 1).copy())
        eng.run(0.0, 100 * dt, dt, SEED)
        fin = eng.get_final(1)
    finally:
        eng.close()
    np.testing.assert_allclose(fin["r"][:, 0], g["x"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(fin["v"][:, 0], g["v"], rtol=1e-8, atol=1e-12)


def test_iesh_golden():
    g = np.load(GOLDEN / "iesh_small.npz")
    n = g["r0"].shape[0]
    wl = WL.newns_anderson_iesh(n, nstates=20, nelectrons=10, z0=3.5)
    np.testing.assert_array_equal(wl["r0"], g["r0"])
    eng = C.iesh_newns_anderson(L, wl, n, L.PREC_FP64, max_hops=16)
    try:
        eng.set_initial(np.ascontiguousarray(g["r0"]), np.ascontiguousarray(g["v0"]))
        eng.run(0.0, 200 * wl["dt"], wl["dt"], SEED)
        fin = eng.get_final_iesh(20, 10)
        log = eng.get_hop_log(16)
    finally:
        eng.close()
    np.testing.assert_array_equal(fin["state"], g["state"])
    np.testing.assert_array_equal(log, g["hop_log"])
    np.testing.assert_allclose(fin["r"], g["r"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(fin["v"], g["v"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(fin["psi"], g["psi_re"] + 1j * g["psi_im"], atol=1e-8)
    np.testing.assert_allclose(fin["energy"], g["energy"], rtol=1e-10, atol=1e-10)
