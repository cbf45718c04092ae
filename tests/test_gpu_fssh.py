"""GPU parity of the FSSH ensemble kernels against the CPU oracle.

Plain FP64 path: bit-identical final phase-space points, density matrices,
states and hop sequences (the oracle and the kernels evaluate the same
operations in the same order).  Fast FP32 path: ensemble observables
within the stated tolerance of the FP64 oracle.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from nqcd_gb300 import _lib as L

pytestmark = pytest.mark.gpu

TULLY = {1: (0.01, 1.6, 0.005, 1.0), 2: (0.1, 0.28, 0.015, 0.06, 0.05), 3: (6e-4, 0.1, 0.9)}


def make_cfg(model, params, ndof, masses, ntraj, precision=L.PREC_FP64, rescaling=0, init_kind=1, init_state=0,
             bath=None, save_stride=0, max_hops=16):
    cfg = L.nqcd_config()
    cfg.method = L.METHOD_FSSH
    cfg.model = model
    cfg.precision = precision
    cfg.rescaling = rescaling
    cfg.ndofs = 1
    cfg.natoms = ndof
    cfg.nstates = 2
    p = np.asarray(params, dtype=np.float64)
    m = np.ascontiguousarray(np.broadcast_to(np.asarray(masses, np.float64), (ndof,)))
    keep = [p, m]
    cfg.nparams = len(p)
    cfg.params = L.dptr(p)
    cfg.masses = L.dptr(m)
    if bath is not None:
        c, w = (np.ascontiguousarray(x, dtype=np.float64) for x in bath)
        keep += [c, w]
        cfg.nbath = ndof
        cfg.bath_a = L.dptr(c)
        cfg.bath_b = L.dptr(w)
    cfg.ntraj_max = ntraj
    cfg.init_kind = init_kind
    cfg.init_state = init_state
    cfg.save_stride = save_stride
    cfg.max_hops = max_hops
    cfg.gap_fp64 = 1e-3
    return cfg, keep


def run_engine(cfg, keep, r0, v0, t0, t1, dt, seed, ndof):
    eng = L.Engine(cfg, keep)
    try:
        eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0))
        sc = np.zeros(4)
        pc = np.zeros(100000)
        out, st = eng.run(t0, t1, dt, seed, scattering=sc, popcorr=pc)
        fin = eng.get_final(ndof)
        fin["hop_log"] = eng.get_hop_log(cfg.max_hops) if cfg.max_hops else None
        fin["scatter"] = sc
        fin["popcorr"] = pc[: out.nsave * 4].reshape(out.nsave, 4)
        fin["stats"] = st
        return fin
    finally:
        eng.close()


def assert_bitwise(eng, orc, ntraj):
    np.testing.assert_array_equal(eng["state"], orc["state"])
    np.testing.assert_array_equal(eng["nhops"], orc["nhops"])
    np.testing.assert_array_equal(eng["nfrustrated"], orc["nfrustrated"])
    np.testing.assert_array_equal(eng["nsteps"], orc["nsteps"])
    np.testing.assert_array_equal(eng["hop_log"], orc["hop_log"])
    np.testing.assert_array_equal(eng["r"], orc["r"])
    np.testing.assert_array_equal(eng["v"], orc["v"])
    np.testing.assert_array_equal(eng["sig_re"], orc["sigma"].real)
    np.testing.assert_array_equal(eng["sig_im"][:, 0, 1], orc["sigma"].imag[:, 0, 1])
    np.testing.assert_array_equal(eng["energy"], orc["energy"])


@pytest.mark.parametrize("model,rescaling,p0", [(1, 0, 10.0), (2, 0, 16.0), (3, 1, 8.0), (1, 2, 12.0)])
def test_tully_fp64_bitwise(model, rescaling, p0):
    ntraj, m = 512, 2000.0
    rng = np.random.default_rng(model * 10 + rescaling)
    r0 = np.full((ntraj, 1), -10.0)
    v0 = (p0 + rng.uniform(-2, 2, (ntraj, 1))) / m
    cfg, keep = make_cfg(model, TULLY[model], 1, m, ntraj, rescaling=rescaling)
    t1 = 3000.0 if model == 1 else 2000.0
    eng = run_engine(cfg, keep, r0, v0, 0.0, t1, 1.0, 1234, 1)
    orc = O.run_fssh(model=model, params=TULLY[model], ndof=1, mass=m, r0=r0, v0=v0, t0=0.0, t1=t1, dt=1.0,
                     seed=1234, rescaling=rescaling, init_kind=1, init_state=0, max_hops=16)
    assert orc["nhops"].sum() > 0  # the test exercises hops
    assert_bitwise(eng, orc, ntraj)
    np.testing.assert_allclose(eng["scatter"], orc["scatter"], rtol=0, atol=1e-15)


def test_tully_fp64_short_step_remainder():
    # a tspan that is not a multiple of dt: the last step is shortened and
    # times are snapped exactly as the reference integrator does
    ntraj, m = 64, 2000.0
    r0 = np.full((ntraj, 1), -5.0)
    v0 = np.linspace(10, 30, ntraj).reshape(ntraj, 1) / m
    cfg, keep = make_cfg(1, TULLY[1], 1, m, ntraj)
    eng = run_engine(cfg, keep, r0, v0, 0.0, 777.7, 0.35, 99, 1)
    orc = O.run_fssh(model=1, params=TULLY[1], ndof=1, mass=m, r0=r0, v0=v0, t0=0.0, t1=777.7, dt=0.35, seed=99)
    assert_bitwise(eng, orc, ntraj)


def spin_boson_case(ntraj, nmodes=100, seed=5):
    wc, alpha, beta = 2.5, 0.1, 5.0
    j = np.arange(1, nmodes + 1)
    w = -wc * np.log(1 - j / (nmodes + 1))
    c = np.sqrt(alpha * wc / (nmodes + 1)) * w
    rng = np.random.default_rng(seed)
    sx = np.sqrt(1 / (2 * w * np.tanh(beta * w / 2)))
    sv = np.sqrt(w / (2 * np.tanh(beta * w / 2)))
    r0 = rng.standard_normal((ntraj, nmodes)) * sx
    v0 = rng.standard_normal((ntraj, nmodes)) * sv
    return w, c, r0, v0


def test_spinboson_fp64_bitwise():
    ntraj, nm = 96, 100
    w, c, r0, v0 = spin_boson_case(ntraj, nm)
    params = (0.0, 1.0)
    cfg, keep = make_cfg(L.MODEL_SPINBOSON, params, nm, 1.0, ntraj, init_kind=2, init_state=0, bath=(c, w),
                         save_stride=2)
    eng = run_engine(cfg, keep, r0, v0, 0.0, 5.0, 0.05, 77, nm)
    orc = O.run_fssh(model=10, params=params, ndof=nm, mass=1.0, r0=r0, v0=v0, t0=0.0, t1=5.0, dt=0.05, seed=77,
                     init_kind=2, init_state=0, bath_c=c, bath_w2=w * w, save_stride=2)
    assert_bitwise(eng, orc, ntraj)
    np.testing.assert_allclose(eng["popcorr"] / ntraj * ntraj, orc["popcorr"], rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("model,rescaling,p0", [(1, 0, 10.0), (2, 1, 12.0), (3, 2, 15.0), (2, 0, 25.0)])
def test_tully_fp32_observables(model, rescaling, p0):
    # fast path (FP32 step loop with Kahan-compensated position and velocity):
    # scattering probabilities within 3 sigma of the FP64 result, every
    # rescaling mode (standard, velocity inversion, none)
    ntraj, m = 8192, 2000.0
    r0 = np.full((ntraj, 1), -10.0)
    v0 = np.full((ntraj, 1), p0 / m)
    cfg64, k64 = make_cfg(model, TULLY[model], 1, m, ntraj, rescaling=rescaling)
    cfg32, k32 = make_cfg(model, TULLY[model], 1, m, ntraj, precision=L.PREC_FP32, rescaling=rescaling)
    a = run_engine(cfg64, k64, r0, v0, 0.0, 3000.0, 1.0, 42, 1)
    b = run_engine(cfg32, k32, r0, v0, 0.0, 3000.0, 1.0, 42, 1)
    p = a["scatter"]
    sig = np.sqrt(np.maximum(p * (1 - p), 1e-4) / ntraj)
    assert np.all(np.abs(a["scatter"] - b["scatter"]) <= 3 * sig + 1e-12), (a["scatter"], b["scatter"])
    # same random stream: almost every trajectory takes the same hop sequence
    same = np.mean(a["state"] == b["state"])
    assert same > 0.97


@pytest.mark.parametrize("precision", [L.PREC_FP32, L.PREC_FP32_KAHAN])
@pytest.mark.parametrize("rescaling", [0, 1])
def test_spinboson_fast_observables(precision, rescaling):
    # fast paths: population-difference correlation within 0.01 (1% of its range) of the FP64 path
    # on the same inputs and random stream, and final phase space close to it for most trajectories
    ntraj, nm = 2048, 100
    w, c, r0, v0 = spin_boson_case(ntraj, nm, seed=9)
    cfg64, k64 = make_cfg(L.MODEL_SPINBOSON, (0.0, 1.0), nm, 1.0, ntraj, init_kind=2, bath=(c, w), save_stride=2,
                          rescaling=rescaling)
    cfg32, k32 = make_cfg(L.MODEL_SPINBOSON, (0.0, 1.0), nm, 1.0, ntraj, precision=precision, init_kind=2,
                          bath=(c, w), save_stride=2, rescaling=rescaling)
    a = run_engine(cfg64, k64, r0, v0, 0.0, 10.0, 0.05, 3, nm)
    b = run_engine(cfg32, k32, r0, v0, 0.0, 10.0, 0.05, 3, nm)
    da = a["popcorr"][:, 0] - a["popcorr"][:, 1]
    db = b["popcorr"][:, 0] - b["popcorr"][:, 1]
    assert np.max(np.abs(da - db)) < 0.01, np.max(np.abs(da - db))
    assert a["nhops"].sum() > 0
    same = (a["state"] == b["state"]) & (a["nhops"] == b["nhops"])
    assert same.mean() > 0.95
    np.testing.assert_allclose(b["r"][same], a["r"][same], atol=2e-3, rtol=0)
    np.testing.assert_allclose(b["energy"], a["energy"], rtol=1e-3)


def test_engine_errors():
    cfg, keep = make_cfg(1, TULLY[1], 1, 2000.0, 8)
    eng = L.Engine(cfg, keep)
    try:
        with pytest.raises(L.EngineError) as e:
            eng.run(0.0, 10.0, 1.0, 1)
        assert e.value.code == -7  # NQCD_ERR_STATE: run before set_initial
        r0 = np.zeros((9, 1))
        with pytest.raises(L.EngineError) as e:
            eng.set_initial(r0, r0)
        assert e.value.code == -1  # more trajectories than capacity
        eng.set_initial(np.zeros((8, 1)) - 10, np.full((8, 1), 0.005))
        with pytest.raises(L.EngineError) as e:
            eng.run(0.0, 10.0, -1.0, 1)
        assert e.value.code == -1
    finally:
        eng.close()
    bad = L.nqcd_config()
    bad.method = 99
    with pytest.raises(L.EngineError):
        L.Engine(bad)


def test_per_trajectory_status():
    """nqcd_get_status: non-finite final states flagged per trajectory, and
    the steps each fast-path trajectory integrated with the FP64 electronics
    (every step when gap_fp64 exceeds any gap; none for the NaN trajectory,
    whose gap compares false), summed into nqcd_stats."""
    ntraj, m, nsteps = 512, 2000.0, 200
    r0 = np.full((ntraj, 1), -10.0)
    v0 = np.full((ntraj, 1), 15.0 / m)
    r0[7, 0] = np.nan
    cfg, keep = make_cfg(1, TULLY[1], 1, m, ntraj, precision=L.PREC_FP32)
    cfg.gap_fp64 = 1e9
    eng = L.Engine(cfg, keep)
    try:
        eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0))
        # the run completes and reports the non-finite trajectory as NQCD_ERR_NAN
        out, st = L.nqcd_outputs(), L.nqcd_stats()
        rc = eng.lib.nqcd_run(eng.h, 0.0, float(nsteps), 1.0, 3, ctypes.byref(out), ctypes.byref(st))
        assert rc == L.NQCD_ERR_NAN
        status = eng.get_status()
    finally:
        eng.close()
    expect_nf = np.zeros(ntraj, np.int32)
    expect_nf[7] = 1
    np.testing.assert_array_equal(status["nonfinite"], expect_nf)
    assert st.flagged == 1
    expect_fb = np.full(ntraj, nsteps, np.int32)
    expect_fb[7] = 0
    np.testing.assert_array_equal(status["fp64_steps"], expect_fb)
    assert st.electronics_fp64_steps == expect_fb.sum()
    # spin-boson fast kernel (4 lanes per trajectory), and the plain path (no fallback)
    nm, n2 = 100, 256
    w, c, rs, vs = spin_boson_case(n2, nm, seed=2)
    for prec, fb in ((L.PREC_FP32_KAHAN, 40), (L.PREC_FP64, 0)):
        cfg, keep = make_cfg(L.MODEL_SPINBOSON, (0.0, 1.0), nm, 1.0, n2, precision=prec, init_kind=2, bath=(c, w))
        cfg.gap_fp64 = 1e9
        eng = L.Engine(cfg, keep)
        try:
            eng.set_initial(np.ascontiguousarray(rs), np.ascontiguousarray(vs))
            _, st = eng.run(0.0, 2.0, 0.05, 3)
            status = eng.get_status()
        finally:
            eng.close()
        np.testing.assert_array_equal(status["fp64_steps"], fb)
        np.testing.assert_array_equal(status["nonfinite"], 0)
        assert st.electronics_fp64_steps == fb * n2
