"""Device-side initial-condition sampling (nqcd_sample_initial).

The sampled positions and velocities equal the numpy restatement of the
documented draw (oracle.sample_initial): fixed and uniform draws bit for bit,
normal draws to the rounding of log and cos; a sharded ensemble equals the
single one; moments match the distributions; run_dynamics with
device_sampling equals the host path fed the same initial conditions.
"""
import numpy as np
import pytest

import oracle as O
import nqcd_gb300 as N
from nqcd_gb300 import _lib as L
from test_gpu_fssh import make_cfg, spin_boson_case

pytestmark = pytest.mark.gpu

SPECS_R = [(L.SAMPLE_NORMAL, 0.3, 0.7), (L.SAMPLE_UNIFORM, -2.0, 5.0), (L.SAMPLE_FIXED, 1.25, 0.0),
           (L.SAMPLE_NORMAL, -1.0, 0.0)]
SPECS_V = [(L.SAMPLE_UNIFORM, 0.0, 1.0), (L.SAMPLE_NORMAL, 0.0, 2.5), (L.SAMPLE_NORMAL, 1e3, 1e-3),
           (L.SAMPLE_FIXED, -4.0, 0.0)]


def sb_engine(ntraj, nmodes, traj_offset=0, method=L.METHOD_FSSH):
    w, c, _, _ = spin_boson_case(1, nmodes)
    cfg, keep = make_cfg(L.MODEL_SPINBOSON, (0.0, 1.0), nmodes, 1.0, ntraj, init_kind=2, bath=(c, w))
    cfg.method = method
    cfg.traj_offset = traj_offset
    return L.Engine(cfg, keep)


def sampled(eng, ntraj, pos, vel, seed, nd):
    eng.sample_initial(ntraj, pos, vel, seed)
    eng.run(0.0, 0.0, 1.0, seed)  # no steps: the final state is the initial one
    fin = eng.get_final(nd)
    return fin["r"], fin["v"]


def test_sampler_matches_restatement():
    n, nd, seed = 20000, len(SPECS_R), 0x1234_5678_9ABC
    eng = sb_engine(n, nd)
    try:
        r, v = sampled(eng, n, SPECS_R, SPECS_V, seed, nd)
    finally:
        eng.close()
    ro, vo = O.sample_initial(SPECS_R, SPECS_V, n, seed)
    for x, xo, specs in ((r, ro, SPECS_R), (v, vo, SPECS_V)):
        for d, (kind, a, b) in enumerate(specs):
            if kind == L.SAMPLE_NORMAL:
                np.testing.assert_allclose(x[:, d], xo[:, d], rtol=1e-13, atol=1e-15 * max(abs(a), b, 1.0))
            else:
                np.testing.assert_array_equal(x[:, d], xo[:, d])
    assert np.all((r[:, 1] >= -2.0) & (r[:, 1] < 5.0))
    np.testing.assert_array_equal(r[:, 3], -1.0)  # zero width


def test_sampler_shards_equal_the_single_ensemble():
    n, nd, seed = 4000, len(SPECS_R), 77
    full = sb_engine(n, nd)
    half = sb_engine(n // 2, nd, traj_offset=n // 2)
    try:
        r, v = sampled(full, n, SPECS_R, SPECS_V, seed, nd)
        r2, v2 = sampled(half, n // 2, SPECS_R, SPECS_V, seed, nd)
    finally:
        full.close()
        half.close()
    np.testing.assert_array_equal(r2, r[n // 2:])
    np.testing.assert_array_equal(v2, v[n // 2:])


def test_sampler_moments():
    n, seed = 1_000_000, 5
    specs_r = [(L.SAMPLE_NORMAL, 0.5, 2.0), (L.SAMPLE_UNIFORM, -1.0, 3.0)]
    specs_v = [(L.SAMPLE_NORMAL, 0.0, 1.0), (L.SAMPLE_NORMAL, -3.0, 0.25)]
    eng = sb_engine(n, 2)
    try:
        r, v = sampled(eng, n, specs_r, specs_v, seed, 2)
    finally:
        eng.close()
    se = 1.0 / np.sqrt(n)
    assert abs(r[:, 0].mean() - 0.5) < 5 * 2.0 * se
    assert abs(r[:, 0].std() - 2.0) < 5 * 2.0 * se
    assert abs(r[:, 1].mean() - 1.0) < 5 * (4.0 / np.sqrt(12)) * se
    assert r[:, 1].min() >= -1.0 and r[:, 1].max() < 3.0
    assert abs(v[:, 0].std() - 1.0) < 5 * se
    assert abs(np.mean(v[:, 0] ** 3)) < 5 * np.sqrt(15) * se  # symmetric
    assert abs(v[:, 1].mean() + 3.0) < 5 * 0.25 * se


def test_run_dynamics_device_sampling_equals_host_path():
    # Ehrenfest (no random hops): device-sampled Wigner ensemble vs the host
    # path fed the restated samples
    ntraj, nm = 512, 20
    model = N.SpinBoson(N.OhmicSpectralDensity(2.5, 0.1), nm, 0.0, 1.0)
    sim = N.Simulation[N.Ehrenfest](N.Atoms(np.ones(nm)), model)
    beta = 5.0
    w = np.asarray(model.ωⱼ)
    pos = [N.PositionHarmonicWigner(wj, beta, 1.0) for wj in w]
    vel = [N.VelocityHarmonicWigner(wj, beta, 1.0) for wj in w]
    dist = N.DynamicalDistribution(vel, pos, (1, nm)) * N.PureState(1, N.Diabatic())
    corr = N.PopulationCorrelationFunction(sim, N.Diabatic())
    kw = dict(output=(corr, N.OutputFinal), trajectories=ntraj, dt=0.05, saveat=0.5, seed=21)
    dev = N.run_dynamics(sim, (0.0, 5.0), dist, ensemble_algorithm=N.EnsembleGB300("fp64", device_sampling=True), **kw)
    r0, v0 = O.sample_initial([p.sampler() for p in pos], [v.sampler() for v in vel], ntraj, 21)
    host_dist = N.DynamicalDistribution(v0.reshape(ntraj, 1, nm), r0.reshape(ntraj, 1, nm), (1, nm)) * \
        N.PureState(1, N.Diabatic())
    host = N.run_dynamics(sim, (0.0, 5.0), host_dist, ensemble_algorithm=N.EnsembleGB300("fp64"), **kw)
    name = N.PopulationCorrelationFunction.__name__
    np.testing.assert_allclose(dev[name], host[name], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(dev["OutputFinal"]["r"], host["OutputFinal"]["r"], rtol=1e-9, atol=1e-12)


def test_sampler_argument_errors():
    eng = sb_engine(16, 2)
    try:
        with pytest.raises(L.EngineError):
            eng.sample_initial(16, [(L.SAMPLE_NORMAL, 0.0, -1.0)] * 2, [(L.SAMPLE_FIXED, 0.0, 0.0)] * 2, 1)
        with pytest.raises(L.EngineError):
            eng.sample_initial(16, [(L.SAMPLE_UNIFORM, 1.0, 0.0)] * 2, [(L.SAMPLE_FIXED, 0.0, 0.0)] * 2, 1)
        with pytest.raises(L.EngineError):
            eng.sample_initial(16, [(7, 0.0, 1.0)] * 2, [(L.SAMPLE_FIXED, 0.0, 0.0)] * 2, 1)
        with pytest.raises(L.EngineError):
            eng.sample_initial(17, [(L.SAMPLE_FIXED, 0.0, 0.0)] * 2, [(L.SAMPLE_FIXED, 0.0, 0.0)] * 2, 1)
    finally:
        eng.close()
