"""GPU parity of Ehrenfest dynamics (NQCD_METHOD_EHRENFEST).

Simulation{Ehrenfest} runs the FSSH integrator (BABwithTsit5,
bab_electronics.jl:61-91) with the mean-field force of the step's initial
density matrix (ehrenfest.jl:50-68) and no hopping.  Plain FP64 path:
bit-identical to the CPU oracle (positions, velocities, density matrices,
energies) for Tully models 1-3 and the spin-boson model, population
correlation and population-resolved scattering to rounding of the sums.
Fast paths: per-trajectory agreement with the plain path (Ehrenfest has no
random hops, so every trajectory is comparable).
"""
import numpy as np
import pytest

import oracle as O
import nqcd_gb300 as N
from nqcd_gb300 import _lib as L
from test_gpu_fssh import TULLY, make_cfg, run_engine, spin_boson_case

pytestmark = pytest.mark.gpu


def ehrenfest_cfg(*args, **kwargs):
    cfg, keep = make_cfg(*args, **kwargs)
    cfg.method = L.METHOD_EHRENFEST
    return cfg, keep


def assert_bitwise_ehrenfest(eng, orc):
    np.testing.assert_array_equal(eng["r"], orc["r"])
    np.testing.assert_array_equal(eng["v"], orc["v"])
    np.testing.assert_array_equal(eng["sig_re"], orc["sigma"].real)
    np.testing.assert_array_equal(eng["sig_im"][:, 0, 1], orc["sigma"].imag[:, 0, 1])
    np.testing.assert_array_equal(eng["energy"], orc["energy"])
    np.testing.assert_array_equal(eng["nhops"], 0)


@pytest.mark.parametrize("model,p0", [(1, 12.0), (2, 20.0), (3, 10.0)])
def test_ehrenfest_fp64_bitwise_tully(model, p0):
    ntraj, m = 256, 2000.0
    rng = np.random.default_rng(model)
    r0 = np.full((ntraj, 1), -9.0) + 0.5 * rng.standard_normal((ntraj, 1))
    v0 = (p0 + 10.0 * rng.random((ntraj, 1))) / m
    cfg, keep = ehrenfest_cfg(model, TULLY[model], 1, m, ntraj)
    eng = run_engine(cfg, keep, r0, v0, 0.0, 2500.0, 1.0, 7, 1)
    orc = O.run_fssh(model=model, params=TULLY[model], ndof=1, mass=m, r0=r0, v0=v0, t0=0.0, t1=2500.0, dt=1.0,
                     seed=7, ehrenfest=True)
    assert_bitwise_ehrenfest(eng, orc)
    # population-resolved scattering: the same per-trajectory sums in another order
    np.testing.assert_allclose(eng["scatter"], orc["scatter"], rtol=1e-12, atol=1e-15)
    assert abs(eng["scatter"].sum() - 1.0) < 1e-9
    assert eng["scatter"][3] > 0.01  # population transferred to the upper state


def test_ehrenfest_fp64_bitwise_spinboson():
    ntraj, nm = 64, 40
    w, c, r0, v0 = spin_boson_case(ntraj, nm, seed=3)
    params = (0.0, 1.0)
    cfg, keep = ehrenfest_cfg(L.MODEL_SPINBOSON, params, nm, 1.0, ntraj, init_kind=2, init_state=0, bath=(c, w),
                              save_stride=4)
    eng = run_engine(cfg, keep, r0, v0, 0.0, 6.0, 0.05, 11, nm)
    orc = O.run_fssh(model=10, params=params, ndof=nm, mass=1.0, r0=r0, v0=v0, t0=0.0, t1=6.0, dt=0.05, seed=11,
                     init_kind=2, init_state=0, bath_c=c, bath_w2=w * w, save_stride=4, ehrenfest=True)
    assert_bitwise_ehrenfest(eng, orc)
    np.testing.assert_allclose(eng["popcorr"], orc["popcorr"], rtol=1e-12, atol=1e-14)
    # <P1 - P2>(t) starts at 1 and relaxes
    d = eng["popcorr"][:, 0] - eng["popcorr"][:, 1]
    assert d[0] == pytest.approx(1.0)
    assert d[-1] < 0.9


@pytest.mark.parametrize("precision", [L.PREC_FP32, L.PREC_FP32_KAHAN])
def test_ehrenfest_fast_matches_plain(precision):
    # Tully 2: each fast trajectory stays close to its plain FP64 twin
    ntraj, m = 2048, 2000.0
    rng = np.random.default_rng(4)
    r0 = np.full((ntraj, 1), -9.0)
    v0 = rng.uniform(10.0, 30.0, (ntraj, 1)) / m
    a = run_engine(*ehrenfest_cfg(2, TULLY[2], 1, m, ntraj), r0, v0, 0.0, 2500.0, 1.0, 5, 1)
    b = run_engine(*ehrenfest_cfg(2, TULLY[2], 1, m, ntraj, precision=precision), r0, v0, 0.0, 2500.0, 1.0, 5, 1)
    np.testing.assert_allclose(b["r"], a["r"], rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(b["sig_re"][:, 1, 1], a["sig_re"][:, 1, 1], atol=2e-4)
    np.testing.assert_allclose(b["scatter"], a["scatter"], atol=2e-4)
    np.testing.assert_allclose(b["energy"], a["energy"], rtol=1e-5)


def test_ehrenfest_spinboson_fast_matches_plain():
    ntraj, nm = 2048, 100
    w, c, r0, v0 = spin_boson_case(ntraj, nm, seed=9)
    params = (0.0, 1.0)
    kw = dict(init_kind=2, bath=(c, w), save_stride=2)
    a = run_engine(*ehrenfest_cfg(L.MODEL_SPINBOSON, params, nm, 1.0, ntraj, **kw), r0, v0, 0.0, 10.0, 0.05, 3, nm)
    b = run_engine(*ehrenfest_cfg(L.MODEL_SPINBOSON, params, nm, 1.0, ntraj, precision=L.PREC_FP32_KAHAN, **kw), r0,
                   v0, 0.0, 10.0, 0.05, 3, nm)
    da = a["popcorr"][:, 0] - a["popcorr"][:, 1]
    db = b["popcorr"][:, 0] - b["popcorr"][:, 1]
    assert np.max(np.abs(da - db)) < 1e-3, np.max(np.abs(da - db))
    np.testing.assert_allclose(b["r"], a["r"], atol=2e-3, rtol=0)
    np.testing.assert_allclose(b["energy"], a["energy"], rtol=1e-3)


def test_ehrenfest_run_dynamics_matches_engine():
    ntraj, m = 128, 2000.0
    sim = N.Simulation[N.Ehrenfest](N.Atoms(m), N.TullyModelOne())
    rng = np.random.default_rng(2)
    r0 = np.full((ntraj, 1, 1), -8.0)
    v0 = rng.uniform(8.0, 25.0, (ntraj, 1, 1)) / m
    dist = N.DynamicalDistribution(v0, r0, (1, 1)) * N.PureState(1, N.Adiabatic())
    res = N.run_dynamics(sim, (0.0, 2000.0), dist, output=(N.OutputStateResolvedScattering1D(sim, "adiabatic"), N.OutputFinal),
                         trajectories=ntraj, dt=1.0, ensemble_algorithm=N.EnsembleGB300("fp64"), seed=3)
    fin = res["OutputFinal"]
    orc = O.run_fssh(model=1, params=TULLY[1], ndof=1, mass=m, r0=r0.reshape(ntraj, 1),
                     v0=v0.reshape(ntraj, 1), t0=0.0, t1=2000.0, dt=1.0, seed=3, ehrenfest=True)
    np.testing.assert_array_equal(fin["r"], orc["r"])
    sc = res["OutputStateResolvedScattering1D"]
    np.testing.assert_allclose(np.concatenate([sc["reflection"], sc["transmission"]]), orc["scatter"], rtol=1e-12,
                               atol=1e-15)
    assert np.all(fin["nhops"] == 0)
