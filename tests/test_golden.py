"""The oracle still reproduces the committed golden fixtures
(tests/golden/*.npz, made by tests/golden/make_golden.py).

FSSH and RPSH come from the C++ oracle and must match bit for bit; MDEF and
IESH call LAPACK through numpy, whose rounding may differ between BLAS
builds, so they match to 1e-9.
"""
import importlib.util
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _maker():
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name", ["fssh_tully1", "fssh_spinboson", "rpsh_mixed"])
def test_oracle_reproduces_golden_bitwise(name):
    ref = np.load(GOLDEN / f"{name}.npz")
    new = getattr(_maker(), name)()
    for k in ref.files:
        np.testing.assert_array_equal(new[k], ref[k], err_msg=k)


@pytest.mark.parametrize("name", ["mdef_small", "iesh_small"])
def test_oracle_reproduces_golden_to_rounding(name):
    ref = np.load(GOLDEN / f"{name}.npz")
    new = getattr(_maker(), name)()
    for k in ref.files:
        if ref[k].dtype.kind in "iu":
            np.testing.assert_array_equal(new[k], ref[k], err_msg=k)
        else:
            np.testing.assert_allclose(new[k], ref[k], rtol=1e-9, atol=1e-11, err_msg=k)
