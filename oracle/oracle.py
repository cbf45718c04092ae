"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (nqcd_oracle.cpp) is an FP64 CPU restatement of NQCDynamics.jl's
ensemble hot path.  Only the test suite, the smoke check and the benchmark's
CPU-baseline leg may use this module; the engine never does.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "_build" / "liboracle.so"

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int32)


class oracle_fssh_args(C.Structure):
    _fields_ = [
        ("model", C.c_int32),
        ("params", C.c_double * 8),
        ("nbath", C.c_int32),
        ("bath_c", DP),
        ("bath_w2", DP),
        ("ndof", C.c_int32),
        ("mass", DP),
        ("rescaling", C.c_int32),
        ("init_kind", C.c_int32),
        ("init_state", C.c_int32),
        ("t0", C.c_double),
        ("t1", C.c_double),
        ("dt", C.c_double),
        ("seed", C.c_uint64),
        ("ntraj", C.c_int64),
        ("traj_offset", C.c_int64),
        ("save_stride", C.c_int32),
        ("nthreads", C.c_int32),
        ("max_hops", C.c_int32),
        ("nbeads", C.c_int32),
        ("beta", C.c_double),
        ("terminate_x", C.c_double),
        ("method", C.c_int32),
    ]


class oracle_fssh_out(C.Structure):
    _fields_ = [
        ("r", DP),
        ("v", DP),
        ("sigma", DP),
        ("state", IP),
        ("hop_log", IP),
        ("nhops", IP),
        ("nfrustrated", IP),
        ("popcorr", DP),
        ("scatter", DP),
        ("nsteps", IP),
        ("energy", DP),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} not built; run __graft_entry__.build()")
        L = C.CDLL(str(LIB))
        L.oracle_fssh_run.argtypes = [C.POINTER(oracle_fssh_args), C.POINTER(oracle_fssh_out)]
        L.oracle_rpsh_run.argtypes = [C.POINTER(oracle_fssh_args), IP, C.c_int32, C.POINTER(oracle_fssh_out)]
        L.oracle_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.oracle_exp.restype = C.c_double
        L.oracle_exp.argtypes = [C.c_double]
        L.oracle_cdiv_real.restype = C.c_double
        L.oracle_cdiv_real.argtypes = [C.c_double] * 4
        L.oracle_uniform.restype = C.c_double
        L.oracle_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32]
        L.oracle_tully.argtypes = [C.c_int32, DP, C.c_double, DP, DP]
        L.oracle_select_new_state.restype = C.c_int32
        L.oracle_select_new_state.argtypes = [DP, C.c_int32, C.c_int32, C.c_double]
        L.oracle_nm_transform.argtypes = [C.c_int32, DP]
        L.oracle_cayley.argtypes = [C.c_int32, C.c_double, C.c_double, DP]
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(DP)


def _i(a):
    return None if a is None else a.ctypes.data_as(IP)


def cdiv_real(a: float, b: float, c: float, d: float) -> float:
    """real((a + ib) / (c + id)) by the restated Julia Complex{Float64} division."""
    return lib().oracle_cdiv_real(a, b, c, d)


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().oracle_philox(c, k, o)
    return list(o)


def exp(x: float) -> float:
    return lib().oracle_exp(float(x))


def uniform(seed, traj, step, stream) -> float:
    return lib().oracle_uniform(seed, traj, step, stream)


def tully(kind: int, params, x: float):
    p = np.zeros(8)
    p[: len(params)] = params
    V = np.zeros(3)
    D = np.zeros(3)
    lib().oracle_tully(kind, _d(p), float(x), _d(V), _d(D))
    return V, D


def select_new_state(cumulative, state: int, u: float) -> int:
    c = np.ascontiguousarray(cumulative, dtype=np.float64)
    return lib().oracle_select_new_state(_d(c), len(c), state, u)


def nm_transform(n: int) -> np.ndarray:
    U = np.zeros(n * n)
    lib().oracle_nm_transform(n, _d(U))
    return U.reshape(n, n, order="F")  # U[j, k]: bead j, mode k


def cayley(n: int, beta: float, dt: float) -> np.ndarray:
    P = np.zeros(n * 4)
    lib().oracle_cayley(n, beta, dt, _d(P))
    return P.reshape(n, 2, 2)


def run_fssh(*, model, params, ndof, mass, r0, v0, t0, t1, dt, seed, rescaling=0, init_kind=1, init_state=0,
             sigma0=None, state0=None, bath_c=None, bath_w2=None, save_stride=0, max_hops=16,
             nthreads=None, traj_offset=0, ehrenfest=False):
    """Run the oracle FSSH (or, with ehrenfest=True, Ehrenfest) ensemble;
    returns a dict of final per-trajectory data."""
    ntraj = r0.shape[0]
    a = oracle_fssh_args()
    a.method = 1 if ehrenfest else 0
    a.model = model
    for q, x in enumerate(params):
        a.params[q] = x
    bc = None if bath_c is None else np.ascontiguousarray(bath_c, dtype=np.float64)
    bw = None if bath_w2 is None else np.ascontiguousarray(bath_w2, dtype=np.float64)
    a.nbath = 0 if bc is None else len(bc)
    a.bath_c = _d(bc)
    a.bath_w2 = _d(bw)
    a.ndof = ndof
    m = np.ascontiguousarray(np.broadcast_to(np.asarray(mass, dtype=np.float64), (ndof,)))
    a.mass = _d(m)
    a.rescaling = rescaling
    a.init_kind = init_kind
    a.init_state = init_state
    a.t0, a.t1, a.dt = t0, t1, dt
    a.seed = seed
    a.ntraj = ntraj
    a.traj_offset = traj_offset
    a.save_stride = save_stride
    a.nthreads = nthreads or os.cpu_count() or 1
    a.max_hops = max_hops
    r = np.ascontiguousarray(r0, dtype=np.float64).reshape(ntraj, -1).copy()
    v = np.ascontiguousarray(v0, dtype=np.float64).reshape(ntraj, -1).copy()
    sig = np.zeros((ntraj, 8))
    if sigma0 is not None:
        s = np.asarray(sigma0, dtype=np.complex128).reshape(ntraj, 2, 2)
        for i in range(2):
            for j in range(2):
                sig[:, 2 * (2 * i + j)] = s[:, i, j].real
                sig[:, 2 * (2 * i + j) + 1] = s[:, i, j].imag
    state = np.zeros(ntraj, np.int32) if state0 is None else np.ascontiguousarray(state0, dtype=np.int32).copy()
    hop_log = np.full((ntraj, max(max_hops, 1), 3), -1, np.int32)
    nh = np.zeros(ntraj, np.int32)
    nf = np.zeros(ntraj, np.int32)
    ns = np.zeros(ntraj, np.int32)
    en = np.zeros((ntraj, 2))
    nsteps_total = 0
    t = t0
    while t < t1:
        h = min(dt, t1 - t)
        t = t + h
        if abs(t - t1) < 100 * np.spacing(max(abs(t), abs(t1))):
            t = t1
        nsteps_total += 1
    nsave = nsteps_total // save_stride + 1 if save_stride > 0 else 0
    pc = np.zeros((max(nsave, 1), 4))
    sc = np.zeros(4)
    o = oracle_fssh_out()
    o.r, o.v, o.sigma, o.state = _d(r), _d(v), _d(sig), _i(state)
    o.hop_log = _i(hop_log) if max_hops > 0 else None
    o.nhops, o.nfrustrated, o.nsteps = _i(nh), _i(nf), _i(ns)
    o.popcorr = _d(pc) if nsave > 0 else None
    o.scatter = _d(sc)
    o.energy = _d(en)
    rc = lib().oracle_fssh_run(C.byref(a), C.byref(o))
    if rc != 0:
        raise RuntimeError(f"oracle_fssh_run failed: {rc}")
    sig_c = np.zeros((ntraj, 2, 2), np.complex128)
    for i in range(2):
        for j in range(2):
            sig_c[:, i, j] = sig[:, 2 * (2 * i + j)] + 1j * sig[:, 2 * (2 * i + j) + 1]
    return dict(r=r, v=v, sigma=sig_c, state=state, hop_log=hop_log, nhops=nh, nfrustrated=nf, nsteps=ns,
                energy=en, popcorr=pc[:nsave] / ntraj if nsave else None, scatter=sc / ntraj)


def run_rpsh(*, model, params, mass, r0, v0, nbeads, beta, t0, t1, dt, seed, rescaling=0, init_kind=1, init_state=0,
             sigma0=None, state0=None, max_hops=16, terminate_x=0.0, nthreads=None, traj_offset=0):
    """Run the oracle ring-polymer FSSH ensemble.  r0, v0: [ntraj][stride] bead
    coordinates (entries past a trajectory's bead count are ignored)."""
    ntraj, stride = r0.shape
    a = oracle_fssh_args()
    a.model = model
    for q, x in enumerate(params):
        a.params[q] = x
    m = np.array([mass], dtype=np.float64)
    a.ndof = 1
    a.mass = _d(m)
    a.rescaling, a.init_kind, a.init_state = rescaling, init_kind, init_state
    a.t0, a.t1, a.dt, a.seed = t0, t1, dt, seed
    a.ntraj, a.traj_offset = ntraj, traj_offset
    a.nthreads = nthreads or os.cpu_count() or 1
    a.max_hops = max_hops
    a.nbeads = stride
    a.beta = beta
    a.terminate_x = terminate_x
    r = np.ascontiguousarray(r0, dtype=np.float64).copy()
    v = np.ascontiguousarray(v0, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbeads, dtype=np.int32)
    sig = np.zeros((ntraj, 8))
    if sigma0 is not None:
        s = np.asarray(sigma0, dtype=np.complex128).reshape(ntraj, 2, 2)
        for i in range(2):
            for j in range(2):
                sig[:, 2 * (2 * i + j)] = s[:, i, j].real
                sig[:, 2 * (2 * i + j) + 1] = s[:, i, j].imag
    state = np.zeros(ntraj, np.int32) if state0 is None else np.ascontiguousarray(state0, dtype=np.int32).copy()
    hop_log = np.full((ntraj, max(max_hops, 1), 3), -1, np.int32)
    nh = np.zeros(ntraj, np.int32)
    nf = np.zeros(ntraj, np.int32)
    ns = np.zeros(ntraj, np.int32)
    en = np.zeros((ntraj, 2))
    sc = np.zeros(4)
    o = oracle_fssh_out()
    o.r, o.v, o.sigma, o.state = _d(r), _d(v), _d(sig), _i(state)
    o.hop_log = _i(hop_log) if max_hops > 0 else None
    o.nhops, o.nfrustrated, o.nsteps = _i(nh), _i(nf), _i(ns)
    o.popcorr = None
    o.scatter = _d(sc)
    o.energy = _d(en)
    rc = lib().oracle_rpsh_run(C.byref(a), _i(nb), stride, C.byref(o))
    if rc != 0:
        raise RuntimeError(f"oracle_rpsh_run failed: {rc}")
    sig_c = np.zeros((ntraj, 2, 2), np.complex128)
    for i in range(2):
        for j in range(2):
            sig_c[:, i, j] = sig[:, 2 * (2 * i + j)] + 1j * sig[:, 2 * (2 * i + j) + 1]
    return dict(r=r, v=v, sigma=sig_c, state=state, hop_log=hop_log, nhops=nh, nfrustrated=nf, nsteps=ns, energy=en,
                scatter=sc / ntraj)


# ---------------------------------------------------------------------------
# Device-side initial-condition sampling (nqcd_sample_initial), restated.
# ---------------------------------------------------------------------------
RNG_INIT_POSITION, RNG_INIT_VELOCITY = 5, 6


def sample_initial(position, velocity, ntraj, seed, traj_offset=0):
    """The engine's sampler (include/nqcd_gpu.h, nqcd_sample_initial) in
    numpy: per trajectory and degree of freedom one Philox4x32-10 block with
    counter (index low, index high, dof, 5 | 6) and key = seed; FIXED a,
    UNIFORM a + (b - a) U(w0, w1), NORMAL a + b sqrt(-2 ln(1 - U(w0, w1)))
    cos(2 pi U(w2, w3)).  Returns r0, v0 of shape (ntraj, ndof)."""
    from mdef_oracle import philox

    traj = np.arange(ntraj, dtype=np.uint64) + np.uint64(traj_offset)
    out = []
    for specs, stream in ((position, RNG_INIT_POSITION), (velocity, RNG_INIT_VELOCITY)):
        x = np.empty((ntraj, len(specs)))
        for d, (kind, a, b) in enumerate(specs):
            if kind == 0:
                x[:, d] = a
                continue
            w = philox((traj & np.uint64(0xFFFFFFFF)).astype(np.uint32), (traj >> np.uint64(32)).astype(np.uint32),
                       np.full(ntraj, d, np.uint32), np.full(ntraj, stream, np.uint32), seed & 0xFFFFFFFF,
                       (seed >> 32) & 0xFFFFFFFF)
            u = (((w[0].astype(np.uint64) << np.uint64(32)) | w[1].astype(np.uint64)) >> np.uint64(11)) * 2.0**-53
            if kind == 2:
                x[:, d] = a + (b - a) * u
            else:
                u2 = (((w[2].astype(np.uint64) << np.uint64(32)) | w[3].astype(np.uint64)) >> np.uint64(11)) * 2.0**-53
                x[:, d] = a + b * (np.sqrt(-2.0 * np.log(1.0 - u)) * np.cos(6.283185307179586 * u2))
        out.append(x)
    return out[0], out[1]
