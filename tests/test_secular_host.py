"""The engine's secular-equation solver (csrc/secular.h) built for the host
(tests/harness/secular_host.cu) and run on the CPU: the roots of the
Newns-Anderson arrowhead Hamiltonians of the MDEF (201 states) and IESH
(80 states) systems against LAPACK, in FP64 and FP32.

* roots to 1e-12 (FP64) and 2e-6 (FP32) of the spectrum's width, impurity
  weights z0^2 to 1e-10 and 1e-4 relative, no unconverged root;
* the resumable form that a lane of the MDEF kernel runs one evaluation at a
  time gives the roots of secular_root bit for bit, from cold and from warm
  starts;
* warm starts from the roots at a nearby level (a step's change of h): about
  one evaluation of f per FP32 root (the Newton step's quadratic error bound
  ends the iteration), the midpoint test and two Newton steps per FP64 root,
  with the roots of a cold solve.
"""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from nqcd_gb300 import workload as WL

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "harness" / "secular_host.cu"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("secular") / "libsecular_host.so"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-shared", str(SRC), "-o", str(out)], check=True,
                   capture_output=True)
    so = C.CDLL(str(out))
    for name, T in (("secular_roots_f32", C.c_float), ("secular_roots_f64", C.c_double)):
        f = getattr(so, name)
        P = C.POINTER(T)
        f.argtypes = [P, P, C.c_int32, T, T, P, P, C.POINTER(C.c_int32), C.c_int32]
        f.restype = C.c_int64
    return so


def solve(lib, eps, V, h, lam0, dtype, resumable):
    eps = np.ascontiguousarray(eps, dtype)
    V2 = np.ascontiguousarray(np.asarray(V, np.float64) ** 2, dtype)
    M = len(eps)
    lam = np.ascontiguousarray(lam0, dtype).copy()
    z2 = np.zeros(M + 1, dtype)
    ev = np.zeros(M + 1, np.int32)
    Lb = abs(h) + abs(float(eps[0])) + abs(float(eps[-1])) + 1.0 + float(V2.sum())
    T = C.c_float if dtype == np.float32 else C.c_double
    f = lib.secular_roots_f32 if dtype == np.float32 else lib.secular_roots_f64
    P = C.POINTER(T)
    nonconv = f(eps.ctypes.data_as(P), V2.ctypes.data_as(P), M, h, Lb, lam.ctypes.data_as(P), z2.ctypes.data_as(P),
                ev.ctypes.data_as(C.POINTER(C.c_int32)), resumable)
    return lam, z2, ev, nonconv


def dense(eps, V, h):
    M = len(eps)
    H = np.zeros((M + 1, M + 1))
    H[0, 0] = h
    H[0, 1:] = H[1:, 0] = V
    H[np.arange(1, M + 1), np.arange(1, M + 1)] = eps
    w, Z = np.linalg.eigh(H)
    return w, Z[0, :] ** 2


SYSTEMS = {
    "mdef201": lambda: WL.newns_anderson_mdef(4, M=200),
    "iesh80": lambda: WL.newns_anderson_iesh(4),
}


@pytest.mark.parametrize("system", list(SYSTEMS))
@pytest.mark.parametrize("dtype,rtol_l,rtol_z", [(np.float64, 1e-12, 1e-10), (np.float32, 2e-6, 1e-4)])
def test_roots_match_lapack(lib, system, dtype, rtol_l, rtol_z):
    wl = SYSTEMS[system]()
    eps, V = np.asarray(wl["eps"]), np.asarray(wl["V"])
    width = eps[-1] - eps[0]
    for h in (-0.4, -0.05, 0.0, 0.03, 0.35):
        w, z2r = dense(eps, V, h)
        # cold start: every interval's midpoint test
        lam, z2, _, nonconv = solve(lib, eps, V, h, np.zeros(len(eps) + 1), dtype, 0)
        assert nonconv == 0
        np.testing.assert_allclose(lam, w, rtol=0, atol=rtol_l * width)
        np.testing.assert_allclose(z2, z2r, rtol=rtol_z, atol=rtol_z * z2r.max() * 1e-3)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_resumable_form_equals_secular_root(lib, dtype):
    wl = SYSTEMS["mdef201"]()
    eps, V = np.asarray(wl["eps"]), np.asarray(wl["V"])
    cold = np.zeros(len(eps) + 1)
    for h in (-0.2, 0.1):
        a = solve(lib, eps, V, h, cold, dtype, 0)
        b = solve(lib, eps, V, h, cold, dtype, 1)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
        # warm starts from the roots at a nearby level
        warm = a[0].astype(np.float64)
        a2 = solve(lib, eps, V, h + 1e-4, warm, dtype, 0)
        b2 = solve(lib, eps, V, h + 1e-4, warm, dtype, 1)
        np.testing.assert_array_equal(a2[0], b2[0])
        np.testing.assert_array_equal(a2[1], b2[1])


@pytest.mark.parametrize("dtype,atol,max_mean", [(np.float64, 1e-12, 3.5), (np.float32, 2e-6, 1.5)])
def test_warm_start_one_evaluation(lib, dtype, atol, max_mean):
    """The level h moves by about 1e-5 per MDEF step at the benchmark's
    velocities: from the previous step's roots an FP32 root takes about one
    evaluation of f (the fast path picks the origin pole from the warm start
    and the quadratic error bound ends the iteration after one step), an FP64
    root its midpoint test and two Newton steps (its tolerance is 2^-52-level),
    and both land where a cold solve does."""
    wl = SYSTEMS["mdef201"]()
    eps, V = np.asarray(wl["eps"]), np.asarray(wl["V"])
    width = eps[-1] - eps[0]
    h0, dh = 0.05, 1e-5
    lam0, _, _, _ = solve(lib, eps, V, h0, np.zeros(len(eps) + 1), dtype, 1)
    lam1, z21, ev, nonconv = solve(lib, eps, V, h0 + dh, lam0.astype(np.float64), dtype, 1)
    assert nonconv == 0
    cold, z2c, evc, _ = solve(lib, eps, V, h0 + dh, np.zeros(len(eps) + 1), dtype, 1)
    np.testing.assert_allclose(lam1, cold, rtol=0, atol=atol * width)
    assert np.mean(ev) < max_mean, np.bincount(ev)
    assert np.mean(ev) < np.mean(evc)
