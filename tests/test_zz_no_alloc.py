"""The allocation-free entry point (nqcd_fssh_spinboson_fp64_noalloc).

It serves callers that cannot allocate device memory while they run; it
must give the same results as the handle API (nqcd_create / nqcd_run), which
for the plain FP64 path means bit for bit.  Two calls in a row check that the
shared fixed scratch array carries nothing from one call into the next.
This file is collected last so that a stop-at-first-failure run has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from nqcd_gb300 import _lib as L
from nqcd_gb300 import workload

pytestmark = pytest.mark.gpu

NMODES = 100


def _bind(lib):
    f = lib.nqcd_fssh_spinboson_fp64_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int32,
                  C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_void_p, C.c_char_p, C.c_int32]
    return f


def run_handle_api(w, c, r0, v0, t1, dt, seed):
    ntraj = r0.shape[0]
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_FSSH, L.MODEL_SPINBOSON, L.PREC_FP64
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, NMODES, 2
    params = np.array([0.0, 1.0])
    masses = np.ones(NMODES)
    cfg.nparams, cfg.params, cfg.masses = 2, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = NMODES, L.dptr(c), L.dptr(w)
    cfg.ntraj_max = ntraj
    cfg.init_kind, cfg.init_state = L.INIT_DIABATIC_PURE, 0
    eng = L.Engine(cfg, [params, masses, c, w])
    try:
        eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0))
        eng.run(0.0, t1, dt, seed)
        return eng.get_final(NMODES)
    finally:
        eng.close()


def run_noalloc(fn, w, c, r0, v0, t1, dt, seed):
    import torch

    dev = torch.device("cuda:0")
    ntraj = r0.shape[0]
    f64 = dict(dtype=torch.float64, device=dev)
    i32 = dict(dtype=torch.int32, device=dev)
    d_c = torch.tensor(c, **f64)
    d_w2 = torch.tensor(w * w, **f64)
    d_m = torch.ones(NMODES, **f64)
    d_r = torch.tensor(np.ascontiguousarray(r0.T), **f64)  # [mode][trajectory]
    d_v = torch.tensor(np.ascontiguousarray(v0.T), **f64)
    d_sig = torch.full((8, ntraj), float("nan"), **f64)
    d_state = torch.full((ntraj,), -1, **i32)
    d_nh = torch.full((ntraj,), -1, **i32)
    d_nf = torch.full((ntraj,), -1, **i32)
    d_ns = torch.full((ntraj,), -1, **i32)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(ntraj, NMODES, d_c.data_ptr(), d_w2.data_ptr(), d_m.data_ptr(), 0.0, 1.0, 0, 0, d_r.data_ptr(),
            d_v.data_ptr(), d_sig.data_ptr(), d_state.data_ptr(), d_nh.data_ptr(), d_nf.data_ptr(), d_ns.data_ptr(),
            0.0, t1, dt, seed, stream, err, 256)
    assert rc == 0, err.value
    torch.cuda.synchronize()
    sig = d_sig.cpu().numpy()
    sig_re = np.stack([sig[0], sig[2], sig[4], sig[6]], axis=1).reshape(ntraj, 2, 2)
    sig_im = np.stack([sig[1], sig[3], sig[5], sig[7]], axis=1).reshape(ntraj, 2, 2)
    return dict(r=d_r.cpu().numpy().T, v=d_v.cpu().numpy().T, sig_re=sig_re, sig_im=sig_im,
                state=d_state.cpu().numpy(), nhops=d_nh.cpu().numpy(), nfrustrated=d_nf.cpu().numpy(),
                nsteps=d_ns.cpu().numpy())


def test_noalloc_matches_handle_api_twice():
    fn = _bind(L.load())
    # two calls in a row with different ensembles: the second must not see the first's scratch
    for ntraj, seed, off in [(1000, 11, 0), (777, 12, 5000)]:
        w, c, r0, v0 = workload.spin_boson_inputs(ntraj, NMODES, traj_offset=off)
        a = run_handle_api(w, c, r0, v0, 4.0, 0.05, seed)
        b = run_noalloc(fn, w, c, r0, v0, 4.0, 0.05, seed)
        assert a["nhops"].sum() > 0
        for key in ("r", "v", "sig_re", "sig_im", "state", "nhops", "nfrustrated", "nsteps"):
            np.testing.assert_array_equal(b[key], a[key], err_msg=key)

