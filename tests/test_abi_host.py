"""C-ABI library and host-side logic, without GPU compute.

* the engine library loads and exports every function include/nqcd_gpu.h declares;
* argument validation answers with the documented error codes before any
  device work (and nqcd_create reports NQCD_ERR_CUDA when no GPU exists);
* the host mirror of the reference API maps simulations to engine configs,
  refuses CPU ensemble algorithms and samples initial conditions as specified.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import nqcd_gb300 as N
from nqcd_gb300 import _lib as L
from nqcd_gb300 import api, workload

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "nqcd_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(nqcd_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    assert set(L.EXPORTED) <= set(names), set(L.EXPORTED) - set(names)


def test_library_exports_every_declared_symbol():
    lib = L.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.nqcd_version() == 111


def _cfg(**kw):
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_FSSH, L.MODEL_TULLY1, L.PREC_FP64
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, 1, 2
    p = np.array([0.01, 1.6, 0.005, 1.0])
    m = np.array([2000.0])
    cfg.nparams, cfg.params, cfg.masses, cfg.ntraj_max = 4, L.dptr(p), L.dptr(m), 16
    cfg.init_kind = L.INIT_ADIABATIC_PURE
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg, [p, m]


@pytest.mark.parametrize("field,value,code", [
    ("method", 99, -6), ("model", 77, -6), ("nstates", 3, -6), ("precision", 5, -1), ("rescaling", 7, -1),
    ("ntraj_max", 0, -1), ("init_state", 2, -1), ("nparams", 2, -1), ("natoms", 2, -6), ("save_stride", -1, -1),
])
def test_create_validates_arguments(field, value, code):
    cfg, keep = _cfg(**{field: value})
    lib = L.load()
    h = C.c_void_p()
    rc = lib.nqcd_create(C.byref(cfg), C.byref(h))
    assert rc == code, (field, rc, lib.nqcd_last_error(None))
    assert not h.value
    assert lib.nqcd_last_error(None)


def test_create_without_gpu_or_with_gpu():
    import torch

    cfg, keep = _cfg()
    lib = L.load()
    h = C.c_void_p()
    rc = lib.nqcd_create(C.byref(cfg), C.byref(h))
    if torch.cuda.is_available():
        assert rc == 0
        lib.nqcd_destroy(h)
    else:
        assert rc == -2 and b"no CUDA device" in lib.nqcd_last_error(None)


def test_null_arguments():
    lib = L.load()
    assert lib.nqcd_create(None, None) == -1
    assert lib.nqcd_run(None, 0.0, 1.0, 1.0, 1, None, None) == -1
    assert lib.nqcd_run_host(None, 1, None, None, 0.0, 1.0, 1.0, 1, None, None) == -1
    assert lib.nqcd_set_initial(None, 1, None, None, None, None, None, None) == -1
    lib.nqcd_destroy(None)  # no-op


def _noalloc(lib):
    f = lib.nqcd_fssh_spinboson_fp64_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int32,
                  C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_void_p, C.c_char_p, C.c_int32]
    return f


_NOALLOC_OK = dict(ntraj=100, nmodes=100, c=8, w2=8, m=8, rescaling=0, state=0, r=8, v=8, sig=8, st=8,
                   t0=0.0, t1=20.0, dt=0.05)


@pytest.mark.parametrize("change,message", [
    (dict(ntraj=0), b"must be positive"),
    (dict(nmodes=0), b"must be positive"),
    (dict(ntraj=1048576 // 100 + 1), b"exceeds the fixed scratch"),
    (dict(c=None), b"null device buffer"),
    (dict(w2=None), b"null device buffer"),
    (dict(m=None), b"null device buffer"),
    (dict(r=None), b"null device buffer"),
    (dict(v=None), b"null device buffer"),
    (dict(sig=None), b"null device buffer"),
    (dict(st=None), b"null device buffer"),
    (dict(rescaling=3), b"rescaling must be"),
    (dict(rescaling=-1), b"rescaling must be"),
    (dict(state=2), b"diabatic_state"),
    (dict(dt=0.0), b"finite t0 <= t1"),
    (dict(dt=float("nan")), b"finite t0 <= t1"),
    (dict(t1=-1.0), b"finite t0 <= t1"),
    (dict(t1=float("inf")), b"finite t0 <= t1"),
    (dict(t0=float("-inf")), b"finite t0 <= t1"),
    (dict(t0=float("nan")), b"finite t0 <= t1"),
    (dict(t1=1.0, dt=1e-300), b"more than 2^31"),
    # a span of 1e4 steps whose clock never moves: 1000 is below half the spacing of doubles at 1e20
    (dict(t0=1e20, t1=1e20 + 1e7, dt=1000.0), b"clock would not advance"),
])
def test_noalloc_rejects_arguments_before_device_work(change, message):
    """Each rejection of the allocation-free entry point answers NQCD_ERR_ARG
    before any device work: the dummy device pointers are never touched."""
    a = dict(_NOALLOC_OK, **change)
    err = C.create_string_buffer(256)
    rc = _noalloc(L.load())(a["ntraj"], a["nmodes"], a["c"], a["w2"], a["m"], 0.0, 1.0, a["rescaling"], a["state"],
                            a["r"], a["v"], a["sig"], a["st"], None, None, None, a["t0"], a["t1"], a["dt"], 1, None,
                            err, 256)
    assert rc == -1, (change, rc, err.value)
    assert message in err.value, err.value


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(L.EngineUnavailable):
        L.load(tmp_path / "absent.so")


def test_ohmic_discretisation_matches_documentation():
    # docs/src/NQCModels/systembathmodels.md:54-59
    d = N.OhmicSpectralDensity(2.5, 0.1)
    w, c = d.discretise(100)
    j = np.arange(1, 101)
    np.testing.assert_allclose(w, -2.5 * np.log(1 - j / 101))
    np.testing.assert_allclose(c, np.sqrt(0.1 * 2.5 / 101) * w)
    w2, c2, r0, v0 = workload.spin_boson_inputs(10, 100)
    np.testing.assert_allclose(w2, w)
    np.testing.assert_allclose(c2, c)


def test_wigner_widths():
    # harmonic Wigner distribution at beta: <x^2> = coth(beta w / 2) / (2 m w), <v^2> = w coth(beta w / 2) / (2 m)
    p = N.PositionHarmonicWigner(1.3, 5.0, 1.0)
    v = N.VelocityHarmonicWigner(1.3, 5.0, 1.0)
    assert abs(p.sigma() ** 2 - 1 / (2 * 1.3 * np.tanh(5 * 1.3 / 2))) < 1e-14
    assert abs(v.sigma() ** 2 - 1.3 / (2 * np.tanh(5 * 1.3 / 2))) < 1e-14
    model = N.SpinBoson(N.OhmicSpectralDensity(2.5, 0.1), 4, 0.0, 1.0)
    pos = [N.PositionHarmonicWigner(w, 5.0, 1.0) for w in model.ωⱼ]
    vel = [N.VelocityHarmonicWigner(w, 5.0, 1.0) for w in model.ωⱼ]
    dist = N.DynamicalDistribution(vel, pos, (1, 4))
    x = dist.sample("r", 200000, np.random.default_rng(0))
    np.testing.assert_allclose(x.std(axis=0), [q.sigma() for q in pos], rtol=0.01)


def test_config_mapping_and_one_based_states():
    sim = N.Simulation[N.FSSH](N.Atoms(2000.0), N.TullyModelTwo(), rescaling="vinversion")
    cfg, keep = api.build_config(sim, N.PureState(2, N.Adiabatic()), 10, N.EnsembleGB300("fp32"), 0)
    assert cfg.model == L.MODEL_TULLY2 and cfg.precision == L.PREC_FP32 and cfg.rescaling == 1
    assert cfg.init_kind == L.INIT_ADIABATIC_PURE and cfg.init_state == 1
    assert [cfg.params[i] for i in range(5)] == [0.1, 0.28, 0.015, 0.06, 0.05]
    with pytest.raises(ValueError):
        api.build_config(sim, N.PureState(3, N.Adiabatic()), 10, N.EnsembleGB300(), 0)
    sb = N.SpinBoson(N.OhmicSpectralDensity(2.5, 0.1), 100, 0.0, 1.0)
    sim2 = N.Simulation[N.FSSH](N.Atoms(np.ones(100)), sb)
    cfg2, _ = api.build_config(sim2, N.PureState(1), 10, N.EnsembleGB300(), 2)
    assert cfg2.init_kind == L.INIT_DIABATIC_PURE and cfg2.nbath == 100 and cfg2.save_stride == 2


def test_cpu_ensemble_algorithms_are_refused():
    sim = N.Simulation[N.FSSH](N.Atoms(2000.0), N.TullyModelOne())
    dist = N.DynamicalDistribution(0.005, -10.0, (1, 1)) * N.PureState(1, N.Adiabatic())
    for alg in (N.EnsembleThreads(), N.EnsembleSerial(), N.EnsembleThreads):
        with pytest.raises(NotImplementedError):
            N.run_dynamics(sim, (0.0, 10.0), dist, output=N.OutputStateResolvedScattering1D(sim, "adiabatic"),
                           trajectories=4, ensemble_algorithm=alg)


def test_unknown_rescaling_and_outputs_rejected():
    # surface_hopping.jl:89-90 throws on an unknown rescaling mode
    with pytest.raises(ValueError):
        N.Simulation[N.FSSH](N.Atoms(2000.0), N.TullyModelOne(), rescaling="bogus")
    with pytest.raises(ValueError):
        N.OutputStateResolvedScattering1D(None, "sideways")


def _iesh_sim(**kw):
    m = N.AndersonHolstein(N.AdsorbateMetal3D(1e-3, 0.2, 1.2, 0.08, 0.3, 0.6), N.TrapezoidalRule(79, -0.5, 0.5),
                           coupling=0.04)
    return N.Simulation[N.AdiabaticIESH](N.Atoms(1837.0), m, **kw), m


def test_metal_models_and_methods_map_to_the_abi():
    sim, m = _iesh_sim(rescaling="vinversion", estimate_probability=False)
    assert m.nstates == 80 and m.nelectrons == 40 and m.kind == L.MODEL_NEWNS_ANDERSON_3D
    eps, w = workload.trapezoidal_rule(79, -0.5, 0.5)
    np.testing.assert_allclose(m.eps, eps)
    np.testing.assert_allclose(m.V, 0.04 * np.sqrt(w))
    cfg, _ = api._metal_config(sim, 16, N.EnsembleGB300("fp32"), 0)
    assert cfg.method == L.METHOD_IESH and cfg.nelectrons == 40 and cfg.rescaling == 1
    assert cfg.exact_hop_probability == 1 and cfg.nbath == 79 and cfg.nstates == 80
    md = N.AndersonHolstein(N.DisplacedHarmonic(0.0294, 1.0, -0.0147), N.ShenviGaussLegendre(200, -0.5, 0.5))
    sim2 = N.Simulation[N.DiabaticMDEF](N.Atoms(1837.0), md, friction_method=N.GaussianBroadening(0.01),
                                        temperature=1 / 1052.6)
    cfg2, _ = api._metal_config(sim2, 16, N.EnsembleGB300("fp64"), 10)
    assert cfg2.method == L.METHOD_MDEF and cfg2.nstates == 201 and cfg2.params[4] == 0.01
    assert cfg2.beta == pytest.approx(1052.6) and cfg2.save_stride == 10


def test_metal_simulation_arguments_are_checked():
    md = N.AndersonHolstein(N.DisplacedHarmonic(0.03, 1.0, -0.015), N.ShenviGaussLegendre(40, -0.5, 0.5))
    with pytest.raises(ValueError):  # friction method required
        N.Simulation[N.DiabaticMDEF](N.Atoms(1837.0), md, temperature=0.001)
    with pytest.raises(NotImplementedError):  # IESH needs the three-dimensional adsorbate
        N.Simulation[N.AdiabaticIESH](N.Atoms(1837.0), md)
    with pytest.raises(ValueError):
        _iesh_sim(rescaling="bogus")
    sim, m = _iesh_sim()
    nuc = N.DynamicalDistribution(np.zeros(3), np.array([0.0, 0.0, 12.0]), (3, 1))
    # iesh.jl:104-113: the distribution's Fermi level must be the model's
    with pytest.raises(ValueError):
        N.run_dynamics(sim, (0.0, 10.0), nuc * N.FermiDiracState(0.1, 1e-3), output=N.OutputFinal, trajectories=2,
                       ensemble_algorithm=N.EnsembleGB300("fp32"))
    with pytest.raises(TypeError):
        N.run_dynamics(sim, (0.0, 10.0), nuc, output=N.OutputFinal, trajectories=2,
                       ensemble_algorithm=N.EnsembleGB300("fp32"))
    with pytest.raises(ValueError):  # time series need saveat
        N.run_dynamics(sim, (0.0, 10.0), nuc * N.FermiDiracState(0.0, 1e-3), output=N.OutputKineticEnergy,
                       trajectories=2, ensemble_algorithm=N.EnsembleGB300("fp32"))


def _rpiesh_cfg(**kw):
    wl = workload.newns_anderson_iesh(4, nstates=20, nelectrons=10)
    P = wl["params"]
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_IESH, L.MODEL_NEWNS_ANDERSON_3D, L.PREC_FP64
    cfg.ndofs, cfg.natoms, cfg.nstates, cfg.nelectrons = 3, 1, 20, 10
    params = np.array([P["kxy"], P["A"], P["a"], P["delta"], P["B"], P["b"]])
    masses = np.array([wl["mass"]])
    eps, V = np.ascontiguousarray(wl["eps"]), np.ascontiguousarray(wl["V"])
    cfg.nparams, cfg.params, cfg.masses = 6, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(eps), L.dptr(eps), L.dptr(V)
    cfg.beta, cfg.ntraj_max, cfg.init_kind, cfg.nbeads_max = wl["beta"], 4, L.INIT_FERMI_DIRAC, 8
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg, [params, masses, eps, V]


@pytest.mark.parametrize("field,value,code", [
    ("method", "ehrenfest_na", -6), ("nbeads_max", 33, -1), ("decoherence_C", 0.1, -6),
    ("beta", 0.0, -1),
])
def test_create_validates_ring_polymer_iesh(field, value, code):
    # RingPolymerSimulation{AdiabaticIESH}: IESH with nbeads_max > 1; checked before any device work
    if value == "ehrenfest_na":
        value = L.METHOD_EHRENFEST_NA
    cfg, keep = _rpiesh_cfg(**{field: value})
    lib = L.load()
    h = C.c_void_p()
    rc = lib.nqcd_create(C.byref(cfg), C.byref(h))
    assert rc == code, (field, rc, lib.nqcd_last_error(None))
    assert not h.value


def test_ring_polymer_iesh_maps_to_the_abi():
    _, m = _iesh_sim()
    sim = N.RingPolymerSimulation[N.AdiabaticIESH](N.Atoms(1837.0), m, 8, temperature=1 / 1052.6,
                                                   rescaling="vinversion")
    cfg, _ = api._metal_config(sim, 16, N.EnsembleGB300("fp64"), 0)
    assert cfg.method == L.METHOD_IESH and cfg.rescaling == 1 and cfg.nelectrons == 40
    with pytest.raises(ValueError):
        N.RingPolymerSimulation[N.AdiabaticIESH](N.Atoms(1837.0), m, 33, temperature=0.001)
    with pytest.raises(NotImplementedError):
        N.RingPolymerSimulation[N.AdiabaticIESH](N.Atoms(1837.0), m, 4, temperature=0.001,
                                                 decoherence=N.DecoherenceCorrectionEDC())
    # per-trajectory arrays in Julia's (ndofs, natoms, nbeads) shape flatten column-major
    r = np.arange(2 * 3 * 4, dtype=float).reshape(2, 3, 1, 4)
    d = N.DynamicalDistribution(r, r, (3, 1, 4))
    flat = d.sample("r", 2, np.random.default_rng(0))
    np.testing.assert_array_equal(flat[1], r[1].reshape(-1, order="F"))
    # the Fermi-Dirac temperature must be the ring polymer's on the GPU path
    dist = d * N.FermiDiracState(0.0, 2e-3)
    with pytest.raises(NotImplementedError):
        N.run_dynamics(sim, (0.0, 1.0), dist, output=N.OutputFinal, trajectories=2,
                       ensemble_algorithm=N.EnsembleGB300("fp64"), dt=0.1)


def _mdef_cfg(**kw):
    wl = workload.newns_anderson_mdef(4, M=40)
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_MDEF, L.MODEL_NEWNS_ANDERSON, L.PREC_FP64
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, 1, 41
    params = np.array([wl["k"], wl["g"], wl["delta"], wl["mu"], wl["sigma"]])
    masses = np.array([wl["mass"]])
    eps, V = np.ascontiguousarray(wl["eps"]), np.ascontiguousarray(wl["V"])
    cfg.nparams, cfg.params, cfg.masses = 5, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = len(eps), L.dptr(eps), L.dptr(V)
    cfg.beta, cfg.ntraj_max = wl["beta"], 4
    keep = [params, masses, eps, V]
    for k, v in kw.items():
        if k in ("eps", "V"):  # replace a bath array
            arr = np.ascontiguousarray(v, dtype=np.float64)
            keep.append(arr)
            setattr(cfg, "bath_a" if k == "eps" else "bath_b", L.dptr(arr))
        else:
            setattr(cfg, k, v)
    return cfg, keep


@pytest.mark.parametrize("which,field,value,code", [
    ("iesh", "nelectrons", 0, -1), ("iesh", "nelectrons", 20, -1), ("iesh", "nstates", 30, -1),
    ("iesh", "precision", L.PREC_FP32_KAHAN, -6), ("iesh", "init_kind", L.INIT_ADIABATIC_PURE, -1),
    ("iesh", "decoherence_C", -1.0, -1), ("iesh", "ndofs", 1, -6), ("iesh", "nparams", 5, -1),
    ("mdef", "beta", 0.0, -1), ("mdef", "nbeads_max", 33, -1), ("mdef", "save_stride", 4, None),
    ("mdef", "nbath", 0, -1), ("mdef", "eps", "descending", -1), ("mdef", "V", "zero", -1),
    ("mdef", "decoherence_C", 0.1, -6), ("mdef", "ndofs", 3, -6),
])
def test_create_validates_metal_models(which, field, value, code):
    # IESH (nqcd_create's IESH block) and MDEF (its MDEF block): every rejection happens before
    # any device work, so on a machine without a GPU an accepted config reports NQCD_ERR_CUDA
    if which == "iesh":
        cfg, keep = _rpiesh_cfg(nbeads_max=0, **{field: value})
    else:
        if value == "descending":
            value = np.linspace(0.5, -0.5, 40)
        elif value == "zero":
            value = np.zeros(40)
        cfg, keep = _mdef_cfg(**{field: value})
    if which == "mdef" and field == "save_stride":
        cfg.nbeads_max = 4  # ring-polymer MDEF reports final states only
        code = -6
    lib = L.load()
    h = C.c_void_p()
    rc = lib.nqcd_create(C.byref(cfg), C.byref(h))
    assert rc == code, (which, field, rc, lib.nqcd_last_error(None))
    assert not h.value


@pytest.mark.parametrize("make", ["mdef", "mdef_rp", "iesh", "iesh_rp"])
def test_valid_metal_configs_pass_validation(make):
    # the unmodified configurations of the validation tests above are accepted: they reach the
    # device (NQCD_ERR_CUDA without a GPU, a handle with one)
    import torch

    if make.startswith("mdef"):
        cfg, keep = _mdef_cfg(nbeads_max=4 if make == "mdef_rp" else 0)
    else:
        cfg, keep = _rpiesh_cfg(nbeads_max=8 if make == "iesh_rp" else 0)
    lib = L.load()
    h = C.c_void_p()
    rc = lib.nqcd_create(C.byref(cfg), C.byref(h))
    if torch.cuda.is_available():
        assert rc == 0
        lib.nqcd_destroy(h)
    else:
        assert rc == -2 and b"no CUDA device" in lib.nqcd_last_error(None), lib.nqcd_last_error(None)


def test_get_final_refuses_orbital_handles():
    """An IESH or EhrenfestNA handle's final state is the orbitals: the
    two-state get_final refuses it before any call into the library (the C
    call would write nelectrons x nstates values per trajectory into 2 x 2
    buffers)."""
    for method in (L.METHOD_IESH, L.METHOD_EHRENFEST_NA):
        eng = object.__new__(L.Engine)
        eng.cfg = L.nqcd_config()
        eng.cfg.method = method
        eng.ntraj = 4
        with pytest.raises(ValueError, match="get_final_iesh"):
            eng.get_final(3)
