"""The IESH FP32 propagator on the fifth-generation tensor cores (tcgen05,
the default where the shape allows: nstates a multiple of 16 up to 80) against
the same path on CUDA cores (nqcd_mapping.iesh_cores = 1), at the benchmark
shape of 80 states and 40 electrons.

The tensor-core products multiply the orbitals as tf32 high + low parts
(2^-22 relative) with the coupling matrix in tf32 (still antisymmetric, so the
effective Hamiltonian stays Hermitian).  So the two paths are not bitwise equal;
they agree to FP32-level tolerance: the same hop sequences in almost every
trajectory, positions and velocities to 1e-4 where the hops agree, orthonormal
orbitals, and ensemble observables within 1 % of the plain FP64 path.
"""
import numpy as np
import pytest

from nqcd_gb300 import _lib as L
from nqcd_gb300 import configs as C
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def run(wl, n, nsteps, precision, cores, seed=13, max_hops=32):
    eng = C.iesh_newns_anderson(L, wl, n, precision, max_hops=max_hops)
    try:
        eng.set_mapping(dict(iesh_cores=cores))
        eng.set_initial(np.ascontiguousarray(wl["r0"]), np.ascontiguousarray(wl["v0"]))
        _, st = eng.run(0.0, nsteps * wl["dt"], wl["dt"], seed)
        fin = eng.get_final_iesh(wl["nstates"], wl["nelectrons"])
        fin["hop_log"] = eng.get_hop_log(max_hops)
        fin["stats"] = st
        return fin
    finally:
        eng.close()


def test_tensor_core_propagator_matches_cuda_cores():
    n, nsteps = 256, 600
    wl = WL.newns_anderson_iesh(n, z0=3.0)
    tc = run(wl, n, nsteps, L.PREC_FP32, 0)
    cc = run(wl, n, nsteps, L.PREC_FP32, 1)
    ref = run(wl, n, nsteps, L.PREC_FP64, 0)
    assert tc["stats"].hops > 0
    # different arithmetic (the cores really differ) ...
    assert not np.array_equal(tc["psi"], cc["psi"])
    # ... to FP32 tolerance
    same = np.array([np.array_equal(a[a[:, 0] >= 0], b[b[:, 0] >= 0]) for a, b in zip(tc["hop_log"], cc["hop_log"])])
    print("hop sequences equal:", same.mean(), "max |psi| diff:", np.abs(tc["psi"] - cc["psi"])[same].max())
    assert same.mean() > 0.9
    np.testing.assert_allclose(tc["r"][same], cc["r"][same], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(tc["v"][same], cc["v"][same], rtol=1e-3, atol=1e-7)
    for t in range(n):
        g = tc["psi"][t].conj().T @ tc["psi"][t]
        assert np.abs(g - np.eye(wl["nelectrons"])).max() < 2e-4, t
    # ensemble means against the plain FP64 path
    for key in ("r", "v"):
        np.testing.assert_allclose(tc[key][:, 2].mean(), ref[key][:, 2].mean(), rtol=0.01)
    np.testing.assert_allclose(tc["energy"][:, 1].mean(), ref["energy"][:, 1].mean(), rtol=0.01)
    assert abs(tc["nhops"].mean() - ref["nhops"].mean()) <= 3 * ref["nhops"].std() / np.sqrt(n) + 0.05
