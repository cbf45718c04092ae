"""GPU parity of the ring-polymer surface-hopping (RPSH) persistent kernel.

Plain FP64 path: bit-identical to the CPU oracle for uneven bead counts,
termination at |centroid| > L, all rescaling modes.  A batch mixing Tully
models 1-3 in one launch equals the per-model launches trajectory by
trajectory.  Fast path: scattering probabilities within statistical error.
"""
import numpy as np
import pytest

import oracle as O
from nqcd_gb300 import _lib as L

pytestmark = pytest.mark.gpu

TULLY = {1: (0.01, 1.6, 0.005, 1.0), 2: (0.1, 0.28, 0.015, 0.06, 0.05), 3: (6e-4, 0.1, 0.9)}
BMAX = 32
BETA = 1024.0
MASS = 2000.0


def rp_inputs(ntraj, seed, counts=(4, 5, 8, 10, 16, 32)):
    rng = np.random.default_rng(seed)
    nb = rng.choice(np.array(counts, np.int32), ntraj).astype(np.int32)
    p = rng.uniform(8.0, 30.0, ntraj)
    r0 = np.full((ntraj, BMAX), -9.5)
    r0 += 0.05 * rng.standard_normal((ntraj, BMAX))  # some spread so that the internal modes move
    v0 = np.repeat((p / MASS)[:, None], BMAX, axis=1)
    return r0, v0, nb


def make_rp_engine(model, ntraj, precision=L.PREC_FP64, rescaling=0, terminate_x=10.0, max_hops=16, gap_fp64=1e-3):
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision, cfg.rescaling = L.METHOD_RPSH, model, precision, rescaling
    cfg.ndofs, cfg.natoms, cfg.nstates, cfg.nbeads_max = 1, 1, 2, BMAX
    p = np.asarray(TULLY[model], np.float64)
    m = np.array([MASS])
    cfg.nparams, cfg.params, cfg.masses = len(p), L.dptr(p), L.dptr(m)
    cfg.beta = BETA
    cfg.ntraj_max = ntraj
    cfg.init_kind, cfg.init_state = L.INIT_ADIABATIC_PURE, 0
    cfg.max_hops = max_hops
    cfg.terminate_x = terminate_x
    cfg.gap_fp64 = gap_fp64
    return L.Engine(cfg, [p, m])


def run_rp(eng, r0, v0, nb, t1, seed, models=None):
    eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0), nbeads=np.ascontiguousarray(nb))
    if models is not None:
        eng.set_trajectory_models(models)
    sc = np.zeros(4)
    out, st = eng.run(0.0, t1, 1.0, seed, scattering=sc)
    fin = eng.get_final(BMAX)
    fin["hop_log"] = eng.get_hop_log(eng.cfg.max_hops)
    fin["scatter"] = sc
    fin["stats"] = st
    return fin


@pytest.mark.parametrize("model,rescaling", [(1, 0), (2, 0), (3, 1), (2, 2)])
def test_rpsh_fp64_bitwise(model, rescaling):
    ntraj = 300
    r0, v0, nb = rp_inputs(ntraj, model * 7 + rescaling)
    eng = make_rp_engine(model, ntraj, rescaling=rescaling)
    try:
        a = run_rp(eng, r0, v0, nb, 4000.0, 31)
    finally:
        eng.close()
    o = O.run_rpsh(model=model, params=TULLY[model], mass=MASS, r0=r0, v0=v0, nbeads=nb, beta=BETA, t0=0.0,
                   t1=4000.0, dt=1.0, seed=31, rescaling=rescaling, terminate_x=10.0, max_hops=16)
    assert o["nhops"].sum() > 0 or model == 3
    assert (o["nsteps"] < 4000).sum() > ntraj // 2  # most trajectories terminate
    np.testing.assert_array_equal(a["nsteps"], o["nsteps"])
    np.testing.assert_array_equal(a["state"], o["state"])
    np.testing.assert_array_equal(a["hop_log"], o["hop_log"])
    np.testing.assert_array_equal(a["nfrustrated"], o["nfrustrated"])
    for t in range(ntraj):  # only the trajectory's own beads are meaningful
        np.testing.assert_array_equal(a["r"][t, : nb[t]], o["r"][t, : nb[t]])
        np.testing.assert_array_equal(a["v"][t, : nb[t]], o["v"][t, : nb[t]])
    np.testing.assert_array_equal(a["sig_re"], o["sigma"].real)
    np.testing.assert_array_equal(a["energy"], o["energy"])
    np.testing.assert_allclose(a["scatter"], o["scatter"], atol=1e-15)


def test_rpsh_mixed_models_one_launch():
    # Tully 1, 2, 3 in contiguous blocks of one launch; the Philox counter is
    # the global trajectory index, so each block equals an oracle run with that offset
    ntraj, blk = 240, 80
    r0, v0, nb = rp_inputs(ntraj, 5)
    models = np.repeat(np.array([1, 2, 3], np.int32), blk)
    eng = make_rp_engine(1, ntraj)
    try:
        mixed = run_rp(eng, r0, v0, nb, 3000.0, 8, models=models)
    finally:
        eng.close()
    for m in (1, 2, 3):
        s = slice((m - 1) * blk, m * blk)
        o = O.run_rpsh(model=m, params=TULLY[m], mass=MASS, r0=r0[s], v0=v0[s], nbeads=nb[s], beta=BETA, t0=0.0,
                       t1=3000.0, dt=1.0, seed=8, terminate_x=10.0, max_hops=16, traj_offset=(m - 1) * blk)
        np.testing.assert_array_equal(mixed["state"][s], o["state"])
        np.testing.assert_array_equal(mixed["nsteps"][s], o["nsteps"])
        np.testing.assert_array_equal(mixed["hop_log"][s], o["hop_log"])
        for j, t in enumerate(range((m - 1) * blk, m * blk)):
            np.testing.assert_array_equal(mixed["r"][t, : nb[t]], o["r"][j, : nb[t]])


def test_rpsh_fast_observables():
    ntraj = 6000
    r0, v0, nb = rp_inputs(ntraj, 3, counts=(4, 8, 16, 32))
    res = {}
    for prec in (L.PREC_FP64, L.PREC_FP32):
        eng = make_rp_engine(1, ntraj, precision=prec)
        try:
            res[prec] = run_rp(eng, r0, v0, nb, 20000.0, 17)
        finally:
            eng.close()
    a, b = res[L.PREC_FP64], res[L.PREC_FP32]
    p = a["scatter"]
    sig = np.sqrt(np.maximum(p * (1 - p), 1e-4) / ntraj)
    assert np.all(np.abs(a["scatter"] - b["scatter"]) <= 3 * sig + 1e-12), (a["scatter"], b["scatter"])
    assert np.mean(a["state"] == b["state"]) > 0.95
    # a few slow trajectories that hop up without rescaling crawl on the upper
    # surface past t1 in both precisions; the unterminated fractions agree
    assert np.mean(a["nsteps"] >= 20000) < 0.005
    assert abs(np.mean(a["nsteps"] >= 20000) - np.mean(b["nsteps"] >= 20000)) <= 0.002
    # termination time agrees to a few steps for trajectories with the same hop history
    same = (a["nhops"] == b["nhops"]) & (a["state"] == b["state"])
    assert np.mean(np.abs(a["nsteps"][same] - b["nsteps"][same]) <= 2) > 0.95


@pytest.mark.parametrize("model,rescaling", [(2, 0), (3, 1)])
def test_rpsh_fast_every_bead_count(model, rescaling):
    """The lane-group fast kernel with bead counts that fill a group (1, 2, 4,
    8, 16, 32) and that leave padding lanes (5, 10): same hop histories as the
    plain path for almost all trajectories, and for those the final centroid
    and ring-polymer energy agree to FP32 accuracy; ring-polymer energy is
    conserved along hop-free trajectories."""
    ntraj = 3000
    r0, v0, nb = rp_inputs(ntraj, 21, counts=(1, 2, 4, 5, 8, 10, 16, 32))
    res = {}
    for prec in (L.PREC_FP64, L.PREC_FP32):
        eng = make_rp_engine(model, ntraj, precision=prec, rescaling=rescaling)
        try:
            res[prec] = run_rp(eng, r0, v0, nb, 6000.0, 5)
        finally:
            eng.close()
    a, b = res[L.PREC_FP64], res[L.PREC_FP32]
    same = (a["nhops"] == b["nhops"]) & (a["state"] == b["state"]) & (a["nfrustrated"] == b["nfrustrated"])
    assert np.mean(same) > 0.95
    for bc in (1, 2, 5, 10, 32):
        assert np.mean(same[nb == bc]) > 0.9, bc
    sel = same & (np.abs(a["nsteps"] - b["nsteps"]) <= 2)
    assert np.mean(sel) > 0.93
    xa = np.array([a["r"][t, : nb[t]].mean() for t in range(ntraj)])
    xb = np.array([b["r"][t, : nb[t]].mean() for t in range(ntraj)])
    assert np.max(np.abs(xa[sel] - xb[sel])) < 0.05
    # initial energies: same initial condition, FP32 bead forces and energies
    np.testing.assert_allclose(b["energy"][:, 0], a["energy"][:, 0], rtol=2e-4, atol=1e-6)
    quiet = sel & (a["nhops"] == 0) & (a["nfrustrated"] == 0)
    drift_a = np.abs(a["energy"][quiet, 1] - a["energy"][quiet, 0])
    drift_b = np.abs(b["energy"][quiet, 1] - b["energy"][quiet, 0])
    assert np.median(drift_b) <= 10 * np.median(drift_a) + 1e-6
    # per-trajectory outputs are written once, at the trajectory's own index
    assert np.all(b["nsteps"] > 0)
    assert np.all(np.isfinite(b["r"][:, 0]))


def test_rpsh_fast_independent_of_queue_order():
    """The fast kernels' results do not depend on which warp integrates a
    trajectory or when: host initial conditions (queues ordered slowest
    first) and device initial conditions (queues in index order) give
    bitwise the same ensemble, and a repeated run reproduces it."""
    torch = pytest.importorskip("torch")
    ntraj = 2000
    r0, v0, nb = rp_inputs(ntraj, 31, counts=(BMAX,))
    eng = make_rp_engine(2, ntraj, precision=L.PREC_FP32, rescaling=1)
    try:
        a = run_rp(eng, r0, v0, nb, 8000.0, 13)
        d_r0 = torch.tensor(np.ascontiguousarray(r0.T), dtype=torch.float64, device="cuda")
        d_v0 = torch.tensor(np.ascontiguousarray(v0.T), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        eng.set_initial_device(ntraj, d_r0.data_ptr(), d_v0.data_ptr())
        sc = np.zeros(4)
        eng.run(0.0, 8000.0, 1.0, 13, scattering=sc)
        b = eng.get_final(BMAX)
        b["scatter"] = sc
        c = run_rp(eng, r0, v0, nb, 8000.0, 13)
    finally:
        eng.close()
    for key in ("r", "v", "state", "nhops", "nfrustrated", "nsteps", "scatter"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
        np.testing.assert_array_equal(a[key], c[key], err_msg=key)
    assert a["nhops"].sum() > 0


def test_rpsh_fast_status_counts_fp64_steps():
    # every step of every trajectory in FP64 electronics: the count equals the trajectory's own step count
    ntraj = 600
    r0, v0, nb = rp_inputs(ntraj, 41, counts=(4, 8, 16, 32, 5, 10))
    eng = make_rp_engine(1, ntraj, precision=L.PREC_FP32, gap_fp64=1e9)
    try:
        fin = run_rp(eng, r0, v0, nb, 4000.0, 9)
        status = eng.get_status()
    finally:
        eng.close()
    np.testing.assert_array_equal(status["fp64_steps"], fin["nsteps"])
    assert fin["stats"].electronics_fp64_steps == int(fin["nsteps"].sum())
    np.testing.assert_array_equal(status["nonfinite"], 0)
