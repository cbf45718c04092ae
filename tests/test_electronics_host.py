"""The fast FSSH electronic sub-integration (csrc/fssh2_traj.h) built for the
host (tests/harness/electronics_host.cu) and run on the CPU against the plain
path's FP64 Tsit5 on the same density matrix and buffer.

The fast path integrates p, q, x, y in FP32 with Tsit5 stages that share the
p/q derivative (dq = -dp) and read G = E0 - E1 and D only; the plain path is
the four-component FP64 Tsit5 that reproduces the reference's
(bab_electronics.jl:61-91).  Checked: one macro step (5 sub-steps of dt/5)
agrees to 2e-6, 400 steps of a slowly varying buffer to 1e-4, the trace p + q
to FP32 rounding, and the same macro step from an energy shift of both levels
is unchanged (the stages read E0 - E1 only).
"""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "harness" / "electronics_host.cu"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("electronics") / "libelectronics_host.so"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-shared", str(SRC), "-o", str(out)], check=True,
                   capture_output=True)
    so = C.CDLL(str(out))
    F, D = C.POINTER(C.c_float), C.POINTER(C.c_double)
    so.electronics_fast_f32.argtypes = [F, C.c_float, C.c_float, F]
    so.electronics_plain_f64.argtypes = [D, C.c_double, C.c_double, D]
    return so


def fast(lib, buf, h, sg):
    b = np.ascontiguousarray(buf, np.float32)
    s = np.ascontiguousarray(sg, np.float32).copy()
    F = C.POINTER(C.c_float)
    lib.electronics_fast_f32(b.ctypes.data_as(F), h, h / 5.0, s.ctypes.data_as(F))
    return s


def plain(lib, buf, h, sg):
    b = np.ascontiguousarray(buf, np.float64)
    s = np.ascontiguousarray(sg, np.float64).copy()
    D = C.POINTER(C.c_double)
    lib.electronics_plain_f64(b.ctypes.data_as(D), h, h / 5.0, s.ctypes.data_as(D))
    return s


def random_sigma(rng):
    # a pure state: sigma = c c^dagger, (p, q, Re sigma_01, Im sigma_01)
    c = rng.standard_normal(2) + 1j * rng.standard_normal(2)
    c /= np.linalg.norm(c)
    s01 = c[0] * np.conj(c[1])
    return np.array([abs(c[0]) ** 2, abs(c[1]) ** 2, s01.real, s01.imag])


def test_one_macro_step_matches_fp64(lib):
    rng = np.random.default_rng(3)
    for _ in range(200):
        E = rng.uniform(-0.05, 0.05, 2)
        dE = rng.uniform(-1e-3, 1e-3, 2)
        D = rng.uniform(-0.02, 0.02)
        buf = [E[0], E[1], D, E[0] + dE[0], E[1] + dE[1], D + rng.uniform(-1e-3, 1e-3)]
        sg = random_sigma(rng)
        h = 0.05 * rng.uniform(0.5, 2.0)
        a = fast(lib, buf, h, sg)
        b = plain(lib, buf, h, sg)
        np.testing.assert_allclose(a, b, rtol=0, atol=2e-6)
        assert abs((a[0] + a[1]) - (sg[0] + sg[1])) < 4e-7


def test_many_steps_track_fp64(lib):
    """400 macro steps with a smoothly moving buffer (the spin-boson run's
    length), the fast state fed back in FP32 and the plain one in FP64."""
    rng = np.random.default_rng(11)
    sg = random_sigma(rng)
    a, b = sg.copy(), sg.copy()
    h = 0.05
    for n in range(400):
        t0, t1 = n * h, (n + 1) * h
        E = lambda t: (0.02 * np.sin(0.3 * t), -0.02 * np.sin(0.3 * t) - 0.03)
        Dd = lambda t: 0.01 * np.cos(0.7 * t)
        buf = [*E(t0), Dd(t0), *E(t1), Dd(t1)]
        a = fast(lib, buf, h, a)
        b = plain(lib, buf, h, b)
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-4)
    assert abs(a[0] + a[1] - 1.0) < 1e-5


def test_fast_step_reads_the_gap_only(lib):
    # shifting both levels by the same amount leaves the fast macro step unchanged
    rng = np.random.default_rng(5)
    sg = random_sigma(rng)
    buf = np.array([0.01, -0.02, 0.004, 0.012, -0.019, 0.0042])
    shift = np.array([0.5, 0.5, 0.0, 0.5, 0.5, 0.0])
    a = fast(lib, buf, 0.05, sg)
    b = fast(lib, buf + shift, 0.05, sg)
    np.testing.assert_allclose(a, b, rtol=0, atol=2e-7)
