"""Batched Jacobi eigensolver (nqcd_eigh_batched) against LAPACK
(numpy.linalg.eigh), the solver the reference's calculators call.

FP64: eigenvalues to 1e-12 of the matrix norm; Z^T A Z diagonal and Z^T Z the
identity to 1e-12; each eigenvector's largest component positive.
FP32: the same to 2e-5 (1e-4 at n = 168).  Also: degenerate spectra, odd orders (bordered
internally), and the arrowhead Newns-Anderson Hamiltonian of the IESH system
whose roots the trajectory kernels take from the secular equation.
"""
import numpy as np
import pytest

import iesh_oracle as IO
from nqcd_gb300 import _lib as L
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def check(A, w, Z, tol):
    norm = np.abs(np.linalg.eigvalsh(A)).max(axis=1)
    wr = np.linalg.eigvalsh(A)
    assert np.all(np.abs(w - wr) <= tol * norm[:, None] + 1e-300)
    n = A.shape[1]
    ZtZ = np.einsum("bij,bik->bjk", Z, Z)
    assert np.abs(ZtZ - np.eye(n)).max() < tol * 10
    D = np.einsum("bij,bik,bkl->bjl", Z, A, Z)
    off = D - np.einsum("bi,ij->bij", np.einsum("bii->bi", D), np.eye(n))
    assert np.abs(off).max() <= tol * 10 * norm.max()
    im = np.abs(Z).argmax(axis=1)
    assert np.all(np.take_along_axis(Z, im[:, None, :], axis=1) > 0)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 16, 33, 80, 120])
def test_eigh_fp64_random(n):
    rng = np.random.default_rng(n)
    B = rng.standard_normal((24, n, n))
    A = 0.5 * (B + B.transpose(0, 2, 1))
    w, Z, sweeps = L.eigh_batched(A)
    check(A, w, Z, 1e-12)
    print(n, "sweeps", sweeps.max())
    assert sweeps.max() < 20


@pytest.mark.parametrize("n,tol", [(16, 2e-5), (80, 2e-5), (168, 1e-4)])
def test_eigh_fp32_random(n, tol):
    # FP32 rotations are orthogonal to a unit in the last place; over about 10 sweeps of n - 1
    # rotations per index the matrix norm drifts by a few units in 1e5 at n = 168
    rng = np.random.default_rng(100 + n)
    B = rng.standard_normal((16, n, n))
    A = 0.5 * (B + B.transpose(0, 2, 1))
    w, Z, _ = L.eigh_batched(A, L.PREC_FP32)
    check(A, w, Z, tol)


def test_eigh_degenerate_and_diagonal():
    n = 12
    A = np.stack([np.eye(n), np.diag(np.repeat([1.0, -2.0, 3.0], 4)), np.zeros((n, n))])
    w, Z, sweeps = L.eigh_batched(A)
    np.testing.assert_array_equal(w[0], np.ones(n))
    np.testing.assert_array_equal(w[1], np.sort(np.repeat([1.0, -2.0, 3.0], 4)))
    np.testing.assert_array_equal(w[2], np.zeros(n))
    assert np.all(sweeps == 0)
    for b in range(3):
        np.testing.assert_allclose(Z[b].T @ Z[b], np.eye(n), atol=1e-15)


def test_eigh_arrowhead_newns_anderson():
    """The IESH system's one-electron Hamiltonian at several heights: the
    Jacobi eigenvalues equal LAPACK's, the values the secular solver of the
    trajectory kernels is tested against."""
    wl = WL.newns_anderson_iesh(4)
    P = wl["params"]
    model = IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                       V=wl["V"])
    z = np.linspace(0.5, 8.0, 16)
    H = model.hamiltonian(np.stack([np.zeros_like(z), np.zeros_like(z), z], axis=1))
    w, Z, _ = L.eigh_batched(H)
    wr, Zr = np.linalg.eigh(H)
    np.testing.assert_allclose(w, wr, rtol=0, atol=1e-13)
    # impurity weights z0^2 of every eigenvector (the force and couplings use them)
    np.testing.assert_allclose(Z[:, 0, :] ** 2, Zr[:, 0, :] ** 2, atol=1e-11)
