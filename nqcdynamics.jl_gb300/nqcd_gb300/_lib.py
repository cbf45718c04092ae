"""ctypes binding of the engine's C ABI (include/nqcd_gpu.h).

The engine has no CPU path: if libnqcd_gb300.so is missing or cannot be
loaded, every call raises EngineUnavailable.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libnqcd_gb300.so"

NQCD_OK = 0
ERRORS = {
    -1: "NQCD_ERR_ARG",
    -2: "NQCD_ERR_CUDA",
    -3: "NQCD_ERR_OOM",
    -4: "NQCD_ERR_TIMEOUT",
    -5: "NQCD_ERR_NAN",
    -6: "NQCD_ERR_UNSUPPORTED",
    -7: "NQCD_ERR_STATE",
}
globals().update({name: code for code, name in ERRORS.items()})  # NQCD_ERR_ARG = -1, ...

METHOD_FSSH, METHOD_RPSH, METHOD_IESH, METHOD_MDEF, METHOD_EHRENFEST, METHOD_EHRENFEST_NA = 1, 2, 3, 4, 5, 6
MODEL_TULLY1, MODEL_TULLY2, MODEL_TULLY3, MODEL_SPINBOSON, MODEL_NEWNS_ANDERSON = 1, 2, 3, 10, 20
MODEL_NEWNS_ANDERSON_3D = 21
MLP_NPARAMS = 4353
PREC_FP64, PREC_FP32, PREC_FP32_KAHAN = 0, 1, 2
RESCALE = {"standard": 0, "vinversion": 1, "off": 2}
INIT_GIVEN, INIT_ADIABATIC_PURE, INIT_DIABATIC_PURE, INIT_FERMI_DIRAC = 0, 1, 2, 3

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int32)


class nqcd_config(C.Structure):
    _fields_ = [
        ("method", C.c_int32),
        ("model", C.c_int32),
        ("precision", C.c_int32),
        ("rescaling", C.c_int32),
        ("ndofs", C.c_int32),
        ("natoms", C.c_int32),
        ("nstates", C.c_int32),
        ("nbeads_max", C.c_int32),
        ("nparams", C.c_int32),
        ("params", DP),
        ("nbath", C.c_int32),
        ("bath_a", DP),
        ("bath_b", DP),
        ("masses", DP),
        ("beta", C.c_double),
        ("ntraj_max", C.c_int64),
        ("init_kind", C.c_int32),
        ("init_state", C.c_int32),
        ("save_stride", C.c_int32),
        ("max_hops", C.c_int32),
        ("terminate_x", C.c_double),
        ("gap_fp64", C.c_double),
        ("traj_offset", C.c_int64),
        ("use_friction_surrogate", C.c_int32),
        ("exact_friction_every", C.c_int32),
        ("nelectrons", C.c_int32),
        ("exact_hop_probability", C.c_int32),
        ("reserved", C.c_int32 * 2),
        ("decoherence_C", C.c_double),
        ("surrogate_tolerance", C.c_double),
    ]


class nqcd_outputs(C.Structure):
    _fields_ = [
        ("scattering", DP),
        ("population_correlation", DP),
        ("observables", DP),
        ("nsave", C.c_int32),
        ("reserved", C.c_int32),
    ]


class nqcd_stats(C.Structure):
    _fields_ = [
        ("traj_steps", C.c_int64),
        ("hops", C.c_int64),
        ("frustrated", C.c_int64),
        ("flagged", C.c_int64),
        ("device_ms", C.c_double),
        ("kernel_ms", C.c_double),
        ("wall_ms", C.c_double),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
        ("kernel_launches", C.c_int32),
        ("reserved", C.c_int32),
        ("exact_friction_evals", C.c_int64),
        ("surrogate_friction_evals", C.c_int64),
        ("unconverged_roots", C.c_int64),
        ("hop_evaluations", C.c_int64),
        ("propagator_terms", C.c_int64),
        ("electronics_fp64_steps", C.c_int64),
        ("surrogate_judged", C.c_int64),
        ("surrogate_rejected", C.c_int64),
        ("surrogate_max_rel_error", C.c_double),
        ("surrogate_mean_rel_error", C.c_double),
        ("overlap_factorizations", C.c_int64),
    ]


class nqcd_sampler(C.Structure):
    """One degree of freedom of a DynamicalDistribution component (nqcd_gpu.h)."""

    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("a", C.c_double), ("b", C.c_double)]


SAMPLE_FIXED, SAMPLE_NORMAL, SAMPLE_UNIFORM = 0, 1, 2


class nqcd_mapping(C.Structure):
    """Launch shapes of the fast kernels (nqcd_gpu.h, nqcd_set_mapping)."""

    _fields_ = [("sb_lanes", C.c_int32), ("sb_block", C.c_int32), ("rp_lanes", C.c_int32 * 4),
                ("iesh_cores", C.c_int32), ("rp_one_launch", C.c_int32), ("iesh_lu_always", C.c_int32)]


RP_LANE_BEADS = (4, 8, 16, 32)  # bead counts of nqcd_mapping.rp_lanes


def mapping(sb_lanes=0, sb_block=0, rp_lanes=None, iesh_cores=0, rp_one_launch=0, iesh_lu_always=0):
    """nqcd_mapping from keyword values; rp_lanes: {bead count: lanes};
    iesh_cores: 0 tensor cores, 1 CUDA cores for the IESH propagator;
    rp_one_launch: 1 serves every bead count from one persistent launch;
    iesh_lu_always: 1 runs the IESH overlap LU every step (0: only where
    the Gram-matrix bound does not settle the hop estimate)."""
    m = nqcd_mapping()
    m.sb_lanes, m.sb_block, m.iesh_cores = int(sb_lanes), int(sb_block), int(iesh_cores)
    m.rp_one_launch, m.iesh_lu_always = int(rp_one_launch), int(iesh_lu_always)
    for q, b in enumerate(RP_LANE_BEADS):
        m.rp_lanes[q] = int((rp_lanes or {}).get(b, 0))
    return m


def samplers(specs):
    """ctypes array of nqcd_sampler from (kind, a, b) triples."""
    arr = (nqcd_sampler * len(specs))()
    for q, (kind, a, b) in enumerate(specs):
        arr[q].kind, arr[q].a, arr[q].b = int(kind), float(a), float(b)
    return arr


EXPORTED = [
    "nqcd_version",
    "nqcd_create",
    "nqcd_set_initial",
    "nqcd_sample_initial",
    "nqcd_set_initial_device",
    "nqcd_run",
    "nqcd_run_host",
    "nqcd_get_final",
    "nqcd_get_hop_log",
    "nqcd_get_status",
    "nqcd_set_trajectory_models",
    "nqcd_set_mapping",
    "nqcd_mdef_evaluate",
    "nqcd_train_friction_mlp",
    "nqcd_mlp_get",
    "nqcd_mlp_set",
    "nqcd_mlp_loss_grad",
    "nqcd_last_error",
    "nqcd_destroy",
    "nqcd_pin_host",
    "nqcd_unpin_host",
    "nqcd_measure_fma_peaks",
    "nqcd_tensor_selftest",
    "nqcd_eigh_batched",
]


def eigh_batched(A, precision=None):
    """Eigenvalues (ascending) and eigenvectors of real symmetric matrices on
    the GPU (nqcd_eigh_batched): A (batch, n, n) -> w (batch, n),
    Z (batch, n, n) with eigenvector o in Z[b, :, o], sweeps (batch,)."""
    A = np.ascontiguousarray(A, np.float64)
    batch, n, _ = A.shape
    w = np.empty((batch, n))
    Zt = np.empty((batch, n, n))
    sw = np.empty(batch, np.int32)
    lib = load()
    rc = lib.nqcd_eigh_batched(PREC_FP64 if precision is None else precision, n, batch, dptr(A), dptr(w), dptr(Zt),
                               iptr(sw))
    if rc:
        raise EngineError(rc, "nqcd_eigh_batched")
    return w, Zt.transpose(0, 2, 1).copy(), sw


class EngineUnavailable(RuntimeError):
    """The CUDA engine library is not built or cannot be loaded."""


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load the engine library (raises EngineUnavailable if absent)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise EngineUnavailable(f"{p} is not built; run __graft_entry__.build() (there is no CPU fallback)")
    try:
        lib = C.CDLL(str(p))
    except OSError as e:  # pragma: no cover - depends on the CUDA runtime being present
        raise EngineUnavailable(f"cannot load {p}: {e}") from e
    lib.nqcd_version.restype = C.c_int
    lib.nqcd_create.argtypes = [C.POINTER(nqcd_config), C.POINTER(C.c_void_p)]
    lib.nqcd_set_initial.argtypes = [C.c_void_p, C.c_int64, DP, DP, DP, DP, IP, IP]
    lib.nqcd_set_initial_device.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, IP]
    lib.nqcd_sample_initial.argtypes = [C.c_void_p, C.c_int64, C.POINTER(nqcd_sampler), C.POINTER(nqcd_sampler),
                                        C.c_uint64]
    lib.nqcd_run.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_uint64,
                             C.POINTER(nqcd_outputs), C.POINTER(nqcd_stats)]
    lib.nqcd_run_host.argtypes = [C.c_void_p, C.c_int64, DP, DP, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                  C.POINTER(nqcd_outputs), C.POINTER(nqcd_stats)]
    lib.nqcd_get_final.argtypes = [C.c_void_p, DP, DP, DP, DP, IP, IP, IP, IP, DP]
    lib.nqcd_get_hop_log.argtypes = [C.c_void_p, IP]
    lib.nqcd_get_status.argtypes = [C.c_void_p, IP, IP]
    lib.nqcd_set_trajectory_models.argtypes = [C.c_void_p, IP]
    lib.nqcd_set_mapping.argtypes = [C.c_void_p, C.POINTER(nqcd_mapping)]
    lib.nqcd_tensor_selftest.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.nqcd_eigh_batched.argtypes = [C.c_int32, C.c_int32, C.c_int64, DP, DP, DP, IP]
    lib.nqcd_mdef_evaluate.argtypes = [C.c_void_p, C.c_int64, DP, DP, DP]
    lib.nqcd_train_friction_mlp.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int64, C.c_int32, C.c_int32,
                                            C.c_double, C.c_uint64, DP]
    FP = C.POINTER(C.c_float)
    lib.nqcd_mlp_get.argtypes = [C.c_void_p, FP, DP]
    lib.nqcd_mlp_set.argtypes = [C.c_void_p, FP, DP]
    lib.nqcd_mlp_loss_grad.argtypes = [C.c_void_p, C.c_int64, DP, DP, DP, FP]
    lib.nqcd_last_error.restype = C.c_char_p
    lib.nqcd_last_error.argtypes = [C.c_void_p]
    lib.nqcd_destroy.argtypes = [C.c_void_p]
    lib.nqcd_destroy.restype = None
    lib.nqcd_pin_host.argtypes = [C.c_void_p, C.c_int64]
    lib.nqcd_unpin_host.argtypes = [C.c_void_p]
    lib.nqcd_measure_fma_peaks.argtypes = [DP, DP]
    if path is None:
        _lib = lib
    return lib


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(DP)


def iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(IP)


class Engine:
    """Owns one nqcd_handle."""

    def __init__(self, cfg: nqcd_config, keepalive=()):
        self.lib = load()
        self._keep = list(keepalive)
        h = C.c_void_p()
        rc = self.lib.nqcd_create(C.byref(cfg), C.byref(h))
        if rc != NQCD_OK:
            raise EngineError(rc, self.lib.nqcd_last_error(None).decode())
        self.h = h
        self.cfg = cfg

    def _check(self, rc: int):
        if rc != NQCD_OK:
            raise EngineError(rc, self.lib.nqcd_last_error(self.h).decode())

    def set_initial(self, r0, v0, sig_re=None, sig_im=None, state0=None, nbeads=None):
        ntraj = r0.shape[0]
        self._check(self.lib.nqcd_set_initial(self.h, ntraj, dptr(r0), dptr(v0), dptr(sig_re), dptr(sig_im),
                                              iptr(state0), iptr(nbeads)))
        self.ntraj = ntraj

    def sample_initial(self, ntraj: int, position, velocity, seed: int):
        """Initial conditions sampled on the device; position/velocity are
        sequences of (kind, a, b) per degree of freedom."""
        self._check(self.lib.nqcd_sample_initial(self.h, ntraj, samplers(position), samplers(velocity), seed))
        self.ntraj = ntraj

    def get_status(self):
        """Per-trajectory status of the last run: non-finite flags and FP64
        electronics step counts."""
        nonfinite = np.empty(self.ntraj, np.int32)
        fp64 = np.empty(self.ntraj, np.int32)
        self._check(self.lib.nqcd_get_status(self.h, iptr(nonfinite), iptr(fp64)))
        return dict(nonfinite=nonfinite, fp64_steps=fp64)

    def set_initial_device(self, ntraj: int, d_r0: int, d_v0: int):
        self._check(self.lib.nqcd_set_initial_device(self.h, ntraj, C.c_void_p(d_r0), C.c_void_p(d_v0), None))
        self.ntraj = ntraj

    def run(self, t0, t1, dt, seed, scattering=None, popcorr=None, observables=None):
        out = nqcd_outputs()
        out.scattering = dptr(scattering)
        out.population_correlation = dptr(popcorr)
        out.observables = dptr(observables)
        st = nqcd_stats()
        self._check(self.lib.nqcd_run(self.h, t0, t1, dt, seed, C.byref(out), C.byref(st)))
        return out, st

    def run_host(self, r0, v0, t0, t1, dt, seed, scattering=None, popcorr=None, observables=None):
        """set_initial(r0, v0) + run(...) in one call (nqcd_run_host): on the fast spin-boson
        path the host-to-device copy of r0, v0 overlaps the integration of earlier chunks."""
        ntraj = r0.shape[0]
        out = nqcd_outputs()
        out.scattering = dptr(scattering)
        out.population_correlation = dptr(popcorr)
        out.observables = dptr(observables)
        st = nqcd_stats()
        self._check(self.lib.nqcd_run_host(self.h, ntraj, dptr(r0), dptr(v0), t0, t1, dt, seed, C.byref(out),
                                           C.byref(st)))
        self.ntraj = ntraj
        return out, st

    def get_final(self, ndof: int, nstates: int = 2):
        if self.cfg.method in (METHOD_IESH, METHOD_EHRENFEST_NA):
            # the C call writes the orbitals (nelectrons x nstates per trajectory) there
            raise ValueError("IESH and EhrenfestNA handles: use get_final_iesh(nstates, nelectrons)")
        n = self.ntraj
        r = np.empty((n, ndof))
        v = np.empty((n, ndof))
        sre = np.empty((n, nstates, nstates))
        sim = np.empty((n, nstates, nstates))
        state = np.empty(n, np.int32)
        nh = np.empty(n, np.int32)
        nf = np.empty(n, np.int32)
        ns = np.empty(n, np.int32)
        en = np.empty((n, 2))
        self._check(self.lib.nqcd_get_final(self.h, dptr(r), dptr(v), dptr(sre), dptr(sim), iptr(state),
                                            iptr(nh), iptr(nf), iptr(ns), dptr(en)))
        # (nstates, nstates) per trajectory arrive column-major: transpose to [i, j]
        return dict(r=r, v=v, sig_re=sre.transpose(0, 2, 1).copy(), sig_im=sim.transpose(0, 2, 1).copy(),
                    state=state, nhops=nh, nfrustrated=nf, nsteps=ns, energy=en)

    def get_final_iesh(self, nstates: int, nelectrons: int):
        """IESH final state: orbitals psi (ntraj, nstates, nelectrons) and
        occupations (ntraj, nelectrons) in electron order; r, v (ntraj, 3), or
        (ntraj, nbeads, 3) for a ring polymer."""
        n = self.ntraj
        nb = self.cfg.nbeads_max if self.cfg.nbeads_max > 1 else 1
        r = np.empty((n, 3 * nb))
        v = np.empty((n, 3 * nb))
        pre = np.empty((n, nelectrons, nstates))
        pim = np.empty((n, nelectrons, nstates))
        occ = np.empty((n, nelectrons), np.int32)
        nh = np.empty(n, np.int32)
        nf = np.empty(n, np.int32)
        ns = np.empty(n, np.int32)
        en = np.empty((n, 2))
        self._check(self.lib.nqcd_get_final(self.h, dptr(r), dptr(v), dptr(pre), dptr(pim), iptr(occ),
                                            iptr(nh), iptr(nf), iptr(ns), dptr(en)))
        psi = (pre + 1j * pim).transpose(0, 2, 1).copy()
        if nb > 1:
            r, v = r.reshape(n, nb, 3), v.reshape(n, nb, 3)
        return dict(r=r, v=v, psi=psi, state=occ, nhops=nh, nfrustrated=nf, nsteps=ns, energy=en)

    def mdef_evaluate(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        F = np.empty_like(x)
        G = np.empty_like(x)
        self._check(self.lib.nqcd_mdef_evaluate(self.h, len(x), dptr(x), dptr(F), dptr(G)))
        return F, G

    def train_friction_mlp(self, lo, hi, npoints, epochs, batch, lr, seed):
        loss = C.c_double()
        self._check(self.lib.nqcd_train_friction_mlp(self.h, lo, hi, npoints, epochs, batch, lr, seed,
                                                     C.byref(loss)))
        return loss.value

    def mlp_get(self):
        w = np.empty(MLP_NPARAMS, np.float32)
        meta = np.empty(4)
        self._check(self.lib.nqcd_mlp_get(self.h, w.ctypes.data_as(C.POINTER(C.c_float)), dptr(meta)))
        return w, meta

    def mlp_set(self, w, meta):
        w = np.ascontiguousarray(w, np.float32)
        meta = np.ascontiguousarray(meta, np.float64)
        self._check(self.lib.nqcd_mlp_set(self.h, w.ctypes.data_as(C.POINTER(C.c_float)), dptr(meta)))

    def mlp_loss_grad(self, x, target):
        x = np.ascontiguousarray(x, np.float64)
        t = np.ascontiguousarray(target, np.float64)
        loss = C.c_double()
        g = np.empty(MLP_NPARAMS, np.float32)
        self._check(self.lib.nqcd_mlp_loss_grad(self.h, len(x), dptr(x), dptr(t), C.byref(loss),
                                                g.ctypes.data_as(C.POINTER(C.c_float))))
        return loss.value, g

    def set_mapping(self, m):
        """Launch shapes for the following runs (nqcd_mapping or a dict of mapping() keywords)."""
        if isinstance(m, dict):
            m = mapping(**m)
        self._check(self.lib.nqcd_set_mapping(self.h, C.byref(m)))

    def set_trajectory_models(self, models):
        self._check(self.lib.nqcd_set_trajectory_models(self.h, iptr(np.ascontiguousarray(models, np.int32))))

    def get_hop_log(self, max_hops: int):
        log = np.empty((self.ntraj, max_hops, 3), np.int32)
        self._check(self.lib.nqcd_get_hop_log(self.h, iptr(log)))
        return log

    def close(self):
        if getattr(self, "h", None):
            self.lib.nqcd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def measure_fma_peaks() -> tuple[float, float]:
    lib = load()
    a, b = C.c_double(), C.c_double()
    rc = lib.nqcd_measure_fma_peaks(C.byref(a), C.byref(b))
    if rc != NQCD_OK:
        raise EngineError(rc, lib.nqcd_last_error(None).decode())
    return a.value, b.value
