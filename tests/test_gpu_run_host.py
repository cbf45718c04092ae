"""nqcd_run_host: set_initial + run in one call, the host-to-device copy of the
initial conditions overlapping the integration of earlier trajectory chunks on
the fast spin-boson path.  Its results equal those of the two calls bit for
bit (every block integrates the same trajectories and writes the same
partial-sum rows), on ensembles that split into ragged chunks, with both lane
groups, for Ehrenfest, and on the configurations that take the two calls in
turn (plain FP64, Tully, given electronic states).  A later nqcd_run repeats
the run from the same initial conditions.
"""
import numpy as np
import pytest

from nqcd_gb300 import _lib as L
from nqcd_gb300 import configs as C
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu

DT, T1 = 0.05, 2.0
NSAVE = int(round(T1 / DT)) // 2 + 1


def spinboson(n, prec, method=None, lanes=0):
    w, c, r0, v0 = WL.spin_boson_inputs(n, 100)
    eng = C.spinboson_fssh(L, w, c, n, 100, prec, save_stride=2, method=method)
    if lanes:
        eng.set_mapping(dict(sb_lanes=lanes, sb_block=128))
    return eng, np.ascontiguousarray(r0), np.ascontiguousarray(v0)


def results(eng, st, pc, sc=None):
    fin = eng.get_final(100)
    out = dict(pc=pc.copy(), r=fin["r"], v=fin["v"], state=fin["state"], nhops=fin["nhops"], energy=fin["energy"],
               sig_re=fin["sig_re"], traj_steps=st.traj_steps, hops=st.hops)
    if sc is not None:
        out["sc"] = sc.copy()
    return out


def assert_same(a, b):
    for k in a:
        np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]), err_msg=k)


@pytest.mark.parametrize("n,prec,method,lanes", [
    (1000, L.PREC_FP32_KAHAN, None, 0),     # 32 blocks of 32 trajectories: 8 chunks, the last one ragged
    (77, L.PREC_FP32_KAHAN, None, 0),       # fewer blocks than chunks
    (4099, L.PREC_FP32, None, 0),           # FP64 accumulators
    (1000, L.PREC_FP32_KAHAN, None, 8),     # 8 lanes per trajectory
    (1000, L.PREC_FP32_KAHAN, L.METHOD_EHRENFEST, 0),
])
def test_run_host_equals_set_initial_and_run(n, prec, method, lanes):
    eng, r0, v0 = spinboson(n, prec, method, lanes)
    try:
        sc = np.zeros(4)
        pc = np.zeros(NSAVE * 4)
        eng.set_initial(r0, v0)
        _, st = eng.run(0.0, T1, DT, 5, popcorr=pc, scattering=sc)
        a = results(eng, st, pc, sc)
        pc[:] = 0.0
        sc[:] = 0.0
        _, st = eng.run_host(r0, v0, 0.0, T1, DT, 5, popcorr=pc, scattering=sc)
        b = results(eng, st, pc, sc)
        assert_same(a, b)
        assert st.h2d_bytes >= r0.nbytes + v0.nbytes
        # the handle keeps the initial conditions: nqcd_run repeats the run
        pc[:] = 0.0
        sc[:] = 0.0
        _, st = eng.run(0.0, T1, DT, 5, popcorr=pc, scattering=sc)
        assert_same(a, results(eng, st, pc, sc))
    finally:
        eng.close()
    assert a["traj_steps"] == n * int(round(T1 / DT))


def test_run_host_fallback_configurations():
    # plain FP64 spin-boson: the two calls in turn, the same results
    eng, r0, v0 = spinboson(300, L.PREC_FP64)
    try:
        pc = np.zeros(NSAVE * 4)
        eng.set_initial(r0, v0)
        _, st = eng.run(0.0, T1, DT, 3, popcorr=pc)
        a = results(eng, st, pc)
        _, st = eng.run_host(r0, v0, 0.0, T1, DT, 3, popcorr=pc)
        assert_same(a, results(eng, st, pc))
    finally:
        eng.close()
    # Tully FSSH on the fast path (not pipelined)
    n = 256
    eng = C.tully_fssh(L, n, L.PREC_FP32_KAHAN)
    try:
        r0, v0 = C.tully_inputs(n)
        r0, v0 = np.ascontiguousarray(r0), np.ascontiguousarray(v0)
        eng.set_initial(r0, v0)
        eng.run(0.0, 500.0, 1.0, 9)
        fa = eng.get_final(1)
        eng.run_host(r0, v0, 0.0, 500.0, 1.0, 9)
        fb = eng.get_final(1)
        np.testing.assert_array_equal(fa["r"], fb["r"])
        np.testing.assert_array_equal(fa["state"], fb["state"])
    finally:
        eng.close()


def test_run_host_rejects_what_set_initial_rejects():
    eng, r0, v0 = spinboson(64, L.PREC_FP32_KAHAN)
    try:
        with pytest.raises(L.EngineError) as e:
            eng.run_host(np.zeros((65, 100)), np.zeros((65, 100)), 0.0, T1, DT, 1)
        assert e.value.code == L.NQCD_ERR_ARG
        with pytest.raises(L.EngineError) as e:
            eng.run_host(r0, v0, 0.0, float("inf"), DT, 1)
        assert e.value.code == L.NQCD_ERR_ARG
    finally:
        eng.close()
