"""GPU parity of EhrenfestNA (NQCD_METHOD_EHRENFEST_NA) on the
three-dimensional Newns-Anderson adsorbate.

Simulation{EhrenfestNA} uses the IESH integrator (VerletwithElectronics) and
Fermi-Dirac initial orbitals with the mean-field force of the orbitals before
each propagation and no hops (ehrenfest_na.jl).  The engine runs it in the
IESH kernel (secular roots, Chebyshev propagator); the oracle with dense
eigendecompositions and the exact propagator.  Plain FP64: positions,
velocities and orbitals to 1e-8, energies to 1e-10, the same initial
occupations; fast FP32: positions and energies to 1e-4, observables to 1e-3 of the plain path.
"""
import numpy as np
import pytest

import iesh_oracle as IO
from nqcd_gb300 import _lib as L
from nqcd_gb300 import workload as WL
from test_gpu_iesh import make_iesh, oracle_model

pytestmark = pytest.mark.gpu


def run_ena(wl, n, nsteps, seed, precision=L.PREC_FP64, save_stride=0):
    eng = make_iesh(wl, n, precision=precision, save_stride=save_stride, method=L.METHOD_EHRENFEST_NA)
    try:
        eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
        obs = np.zeros((nsteps // save_stride + 1) * 4) if save_stride else None
        _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], seed, observables=obs)
        fin = eng.get_final_iesh(wl["nstates"], wl["nelectrons"])
        fin["stats"] = st
        fin["obs"] = None if obs is None else obs.reshape(-1, 4)
        return fin
    finally:
        eng.close()


@pytest.mark.parametrize("nstates,nelectrons,n,nsteps", [(20, 10, 8, 400), (80, 40, 4, 200)])
def test_ehrenfest_na_fp64_matches_oracle(nstates, nelectrons, n, nsteps):
    wl = WL.newns_anderson_iesh(n, nstates=nstates, nelectrons=nelectrons, z0=3.5)
    fin = run_ena(wl, n, nsteps, 3, save_stride=nsteps // 4)
    o = IO.run_iesh(oracle_model(wl), mass=wl["mass"], ne=nelectrons, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"],
                    dt=wl["dt"], nsteps=nsteps, seed=3, ehrenfest_na=True)
    np.testing.assert_array_equal(fin["state"], o["initial_state"])  # occupations never change
    assert fin["stats"].hops == 0 and np.all(fin["nhops"] == 0)
    np.testing.assert_allclose(fin["r"], o["r"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(fin["v"], o["v"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(fin["psi"], o["psi"], atol=1e-8)
    np.testing.assert_allclose(fin["energy"], o["energy"], rtol=1e-10, atol=1e-10)
    # final save point: mean impurity population of the orbitals
    assert fin["obs"][-1, 2] == pytest.approx(o["nimp"].mean(), rel=1e-8)


def test_ehrenfest_na_fp32_matches_fp64():
    n, nsteps = 64, 400
    wl = WL.newns_anderson_iesh(n, nstates=80, nelectrons=40, z0=3.5)
    a = run_ena(wl, n, nsteps, 5, save_stride=50)
    b = run_ena(wl, n, nsteps, 5, precision=L.PREC_FP32, save_stride=50)
    # FP32 orbitals over 400 steps: positions to 1e-4 relative (about 1e-5 seen
    # near the turning point at the surface), observables to 1e-3
    np.testing.assert_array_equal(a["state"], b["state"])
    np.testing.assert_allclose(b["r"], a["r"], rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(b["obs"][:, 2], a["obs"][:, 2], atol=1e-3)
    np.testing.assert_allclose(b["energy"], a["energy"], rtol=1e-4)
