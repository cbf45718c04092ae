"""Fifth-generation tensor cores (tcgen05.mma kind::tf32, accumulator in
tensor memory) through the C ABI's self-test: one 128 x 80 x 80 product, the
shape of the IESH propagator terms, against the float64 product of the same
inputs.  One pass rounds the operands to tf32 (10-bit mantissa); the 3xTF32
split (high and low parts, three products) comes close to fp32 accuracy."""
import ctypes as C

import numpy as np
import pytest

from nqcd_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def test_tcgen05_tf32_products_match_float64():
    lib = L.load()
    f = lib.nqcd_tensor_selftest
    f.restype = C.c_int
    f.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(1)
    A = rng.standard_normal((128, 80)).astype(np.float32)
    B = rng.standard_normal((80, 80)).astype(np.float32)
    ref = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(ref).max()
    errs = {}
    for passes in (1, 3):
        D = np.full((128, 80), np.nan, np.float32)
        rc = f(passes, A.ctypes.data, B.ctypes.data, D.ctypes.data)
        assert rc == 0, rc
        errs[passes] = float(np.abs(D - ref).max() / scale)
    print("relative error: 1 pass", errs[1], "3xTF32", errs[3])
    assert errs[1] < 2e-3
    assert errs[3] < 1e-5
    assert errs[3] < errs[1] / 50
