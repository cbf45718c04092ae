"""Pin the CPU oracle against the reference's own known answers and invariants.

The reference (NQCDynamics.jl) is pure Julia and cannot run here, so the
oracle is checked against the golden vectors, known-answer tests and
invariants its test suite and documentation hold for this path, and against
published algorithm vectors (Philox4x32-10).
"""
import math

import numpy as np
import pytest

import oracle as O

TULLY = {1: (0.01, 1.6, 0.005, 1.0), 2: (0.1, 0.28, 0.015, 0.06, 0.05), 3: (6e-4, 0.1, 0.9)}


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10 (Salmon et al., SC'11)
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_uniform_stream_properties():
    u = np.array([O.uniform(20261203, t, s, 1) for t in range(200) for s in range(50)])
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01 and abs(u.var() - 1 / 12) < 0.005
    # distinct streams and counters give distinct draws
    assert O.uniform(1, 5, 7, 1) != O.uniform(1, 5, 7, 2) != O.uniform(1, 6, 7, 1)


def test_exp_error_bound():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-745, 709, 20000), rng.uniform(-30, 30, 20000), [0.0, 1e-300, -1e-300]])
    for x in xs:
        ref = math.exp(x)
        if ref == 0.0 or not math.isfinite(ref):
            continue
        assert abs(O.exp(x) - ref) <= 2 * math.ulp(ref), x
    assert O.exp(800.0) == math.inf and O.exp(-800.0) == 0.0 and math.isnan(O.exp(float("nan")))


def test_normal_mode_transform_golden_vectors():
    # docs/src/api/RingPolymerArrays/ringpolymerarrays.md:93-133 (n = 4)
    U = O.nm_transform(4)
    to = U.T @ np.ones(4)
    np.testing.assert_allclose(to, [2.0, -8.65956e-17, 0.0, 2.59787e-16], atol=1e-21, rtol=1e-5)
    frm = U @ np.ones(4)
    np.testing.assert_allclose(frm, [1.70711, -0.707107, 0.292893, 0.707107], rtol=1e-5)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 10, 16, 32])
def test_normal_mode_transform_invariants(n):
    # test/Core/ring_polymers.jl:22-27: U'U = I, |det U| = 1, U'SU diagonal with the normal-mode springs
    U = O.nm_transform(n)
    np.testing.assert_allclose(U.T @ U, np.eye(n), atol=1e-13)
    assert abs(abs(np.linalg.det(U)) - 1) < 1e-12
    wn = 2.0
    if n == 1:
        S = np.zeros((1, 1))
    elif n == 2:
        S = np.array([[2.0, -2.0], [-2.0, 2.0]])
    else:
        S = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
        S[0, -1] = S[-1, 0] = -1
    S = S * wn**2 / 2
    lam = (2 * wn * np.sin(np.arange(n) * np.pi / n)) ** 2 / 2
    np.testing.assert_allclose(U.T @ S @ U, np.diag(lam), atol=1e-12 * max(1, lam.max()))


def test_cayley_half_squared_is_full():
    # test/Core/ring_polymers.jl:30-32 and the definition in ring_polymer.jl:71-82
    import scipy.linalg

    for n, beta, dt in [(10, 1.0, 0.1), (4, 1024.0, 1.0), (32, 1024.0, 1.0)]:
        full = O.cayley(n, beta, dt)
        wn = n / beta
        for k in range(n):
            w = 2 * wn * np.sin(k * np.pi / n)
            A = np.array([[0.0, 1.0], [-w * w, 0.0]])
            ref = np.linalg.inv(np.eye(2) - dt * A / 2) @ (np.eye(2) + dt * A / 2)
            np.testing.assert_allclose(full[k], ref, rtol=1e-13, atol=1e-15)
            half = np.real(scipy.linalg.sqrtm(full[k]))
            np.testing.assert_allclose(half @ half, full[k], rtol=1e-10, atol=1e-12)
            # the free-ring-polymer propagator is symplectic: det = 1
            assert abs(np.linalg.det(full[k]) - 1) < 1e-12


def test_select_new_state_known_answers():
    # test/Dynamics/fssh.jl:53-63 (1-based states there, 0-based here)
    assert O.select_new_state([0.0, 1.0], 0, 0.5) == 1
    assert O.select_new_state([0.0, 1.0], 1, 0.5) == 1
    assert O.select_new_state([1.0, 0.0], 1, 0.5) == 0


@pytest.mark.parametrize("kind", [1, 2, 3])
def test_tully_derivative_finite_difference(kind):
    # test/Dynamics/utils.jl:9-62 style consistency of V and dV/dx
    for x in np.linspace(-6, 6, 37):
        _, D = O.tully(kind, TULLY[kind], x)
        h = 1e-6
        Vp, _ = O.tully(kind, TULLY[kind], x + h)
        Vm, _ = O.tully(kind, TULLY[kind], x - h)
        # central differences: O(h^2) truncation, O(h) at Tully 1's x = 0 kink of d2V/dx2
        np.testing.assert_allclose(D, (Vp - Vm) / (2 * h), atol=5e-8)


def test_tully_closed_form_values():
    # Tully, J. Chem. Phys. 93, 1061 (1990)
    V, _ = O.tully(1, TULLY[1], 1.0)
    assert np.allclose(V, [0.01 * (1 - np.exp(-1.6)), 0.005 * np.exp(-1.0), -0.01 * (1 - np.exp(-1.6))], rtol=1e-15)
    V, _ = O.tully(2, TULLY[2], 0.5)
    assert np.allclose(V, [0.0, 0.015 * np.exp(-0.06 * 0.25), -0.1 * np.exp(-0.28 * 0.25) + 0.05], rtol=1e-15)
    V, _ = O.tully(3, TULLY[3], -1.0)
    assert np.allclose(V, [6e-4, 0.1 * np.exp(-0.9), -6e-4], rtol=1e-15)


def test_fssh_total_energy_conserved_tully2():
    # test/Dynamics/fssh.jl:123-133: Tully 2, m = 2000, x = -10, v = 100/2000, dt = 0.1, rtol 1e-2
    n = 64
    r0 = np.full((n, 1), -10.0)
    v0 = np.full((n, 1), 100 / 2000)
    o = O.run_fssh(model=2, params=TULLY[2], ndof=1, mass=2000.0, r0=r0, v0=v0, t0=0.0, t1=500.0, dt=0.1, seed=3)
    assert o["nhops"].sum() > 0
    np.testing.assert_allclose(o["energy"][:, 1], o["energy"][:, 0], rtol=1e-2)


def test_fssh_hop_rescaling_conserves_energy():
    # test/Dynamics/fssh.jl:87-121: an accepted hop changes KE by -dE (rtol 1e-3)
    # through a whole trajectory with hops: total energy drift stays at the integrator level
    n = 256
    r0 = np.full((n, 1), -10.0)
    v0 = np.linspace(9.0, 25.0, n).reshape(n, 1) / 2000
    o = O.run_fssh(model=1, params=TULLY[1], ndof=1, mass=2000.0, r0=r0, v0=v0, t0=0.0, t1=3000.0, dt=1.0, seed=11)
    hopped = o["nhops"] > 0
    assert hopped.sum() > 20
    np.testing.assert_allclose(o["energy"][hopped, 1], o["energy"][hopped, 0], rtol=1e-2)


def test_fssh_frustrated_hops_and_vinversion():
    # test/Dynamics/fssh.jl:65-74: zero momentum -> frustrated, large momentum -> accepted
    n = 128
    r0 = np.full((n, 1), -4.0)
    v0 = np.full((n, 1), 4.5 / 2000)  # too little energy to reach the upper state of Tully 2
    std = O.run_fssh(model=2, params=TULLY[2], ndof=1, mass=2000.0, r0=r0, v0=v0, t0=0.0, t1=1500.0, dt=1.0, seed=5)
    inv = O.run_fssh(model=2, params=TULLY[2], ndof=1, mass=2000.0, r0=r0, v0=v0, t0=0.0, t1=1500.0, dt=1.0, seed=5,
                     rescaling=1)
    off = O.run_fssh(model=2, params=TULLY[2], ndof=1, mass=2000.0, r0=r0, v0=v0, t0=0.0, t1=1500.0, dt=1.0, seed=5,
                     rescaling=2)
    assert std["nfrustrated"].sum() > 0 and std["nhops"].sum() == 0
    assert inv["nfrustrated"].sum() > 0
    assert off["nfrustrated"].sum() == 0 and off["nhops"].sum() > 0


def test_spinboson_diabatic_population_at_symmetric_point():
    # test/Dynamics/fssh.jl:47-51 analogue: symmetric two-level system at R = 0,
    # adiabatic pure state -> diabatic populations 0.5 / 0.5
    n, nm = 4, 10
    w = np.linspace(0.5, 3, nm)
    c = 0.1 * w
    o = O.run_fssh(model=10, params=(0.0, 1.0), ndof=nm, mass=1.0, r0=np.zeros((n, nm)), v0=np.zeros((n, nm)),
                   t0=0.0, t1=0.0, dt=0.1, seed=1, init_kind=1, init_state=0, bath_c=c, bath_w2=w * w, save_stride=1)
    np.testing.assert_allclose(o["popcorr"][0], [0.25, 0.25, 0.25, 0.25], rtol=1e-14)


def test_density_matrix_stays_hermitian_and_normalised():
    n = 32
    r0 = np.full((n, 1), -10.0)
    v0 = np.full((n, 1), 15.0 / 2000)
    o = O.run_fssh(model=1, params=TULLY[1], ndof=1, mass=2000.0, r0=r0, v0=v0, t0=0.0, t1=1200.0, dt=1.0, seed=2)
    s = o["sigma"]
    np.testing.assert_array_equal(s[:, 0, 1], np.conj(s[:, 1, 0]))
    np.testing.assert_allclose(np.trace(s, axis1=1, axis2=2).real, 1.0, atol=1e-8)


def _exact_real_quotient(a, b, c, d):
    from fractions import Fraction as F

    a, b, c, d = map(F, (a, b, c, d))
    return (a * c + b * d) / (c * c + d * d)


def test_complex_division_follows_the_robust_algorithm():
    """real(z / w) as Julia divides Complex{Float64} (Baudin and Smith 2012):
    within a few roundings of the exact quotient for ordinary operands, exactly
    a * (1 / c) for a real denominator, and finite where the textbook formula
    (a c + b d) / (c^2 + d^2) overflows or underflows."""
    rng = np.random.default_rng(5)
    for _ in range(2000):
        a, b, c, d = rng.standard_normal(4) * 10.0 ** rng.integers(-5, 5, 4)
        got = O.cdiv_real(a, b, c, d)
        ex = float(_exact_real_quotient(a, b, c, d))
        # a few roundings of the summands a c and b d (their sum may cancel)
        scale = (abs(a * c) + abs(b * d)) / (c * c + d * d)
        assert abs(got - ex) <= 4 * np.spacing(scale), (a, b, c, d, got, ex)
    for a, b, c in [(0.3, -0.2, 0.7), (-1e-3, 5e-4, 0.999), (0.5, 0.0, 0.5), (0.0, 0.4, 0.6)]:
        assert O.cdiv_real(a, b, c, 0.0) == a * (1.0 / c)
    # pairs near the overflow and underflow thresholds, where the scaling steps act
    for a, b, c, d in [(1e308, 1e308, 1e308, 1e308), (1e-310, 3e-311, 2e-310, -1e-310), (1.0, 1.0, 1e300, 1e-300),
                       (1e-300, 1e-300, 1e-300, 1e-300), (2.0 ** -1000, 1.0, 2.0 ** -1000, 2.0 ** 1000)]:
        got = O.cdiv_real(a, b, c, d)
        ex = float(_exact_real_quotient(a, b, c, d))
        assert math.isfinite(got)
        assert abs(got - ex) <= 4 * np.spacing(abs(ex)) + 2 ** -1074, (a, b, c, d, got, ex)


def test_two_state_density_matrix_diagonal_stays_exactly_real():
    """The oracle carries the full complex 2x2 density matrix through the
    reference's commutator (electronic_dynamics.jl:106-116,
    density_matrix_dynamics.jl:29-33).  Its diagonal stays exactly real: the
    real part of [A, sigma]_ss is (E_s p - D y) - (p E_s - y D), zero in
    floating point.  So real(sigma[m, s] / sigma[s, s]) divides by an exactly
    real sigma[s, s], and the kernels, which carry the diagonal as real
    numbers, divide by (p, 0)."""
    n = 48
    rng = np.random.default_rng(9)
    for kind in (1, 2, 3):
        r0 = np.full((n, 1), -10.0)
        v0 = rng.uniform(8.0, 30.0, (n, 1)) / 2000.0
        for t1 in (700.0, 1500.0, 3000.0):
            o = O.run_fssh(model=kind, params=TULLY[kind], ndof=1, mass=2000.0, r0=r0, v0=v0, t0=0.0, t1=t1, dt=1.0,
                           seed=3)
            assert np.all(o["sigma"][:, 0, 0].imag == 0.0) and np.all(o["sigma"][:, 1, 1].imag == 0.0)
        assert o["nhops"].sum() > 0
    nm = 20
    w = np.linspace(0.1, 3.0, nm)
    c = 0.3 * w
    o = O.run_fssh(model=10, params=(0.0, 1.0), ndof=nm, mass=1.0, r0=rng.standard_normal((n, nm)),
                   v0=rng.standard_normal((n, nm)), t0=0.0, t1=8.0, dt=0.05, seed=4, init_kind=2, init_state=0,
                   bath_c=c, bath_w2=w * w)
    assert o["nhops"].sum() > 0
    assert np.all(o["sigma"][:, 0, 0].imag == 0.0) and np.all(o["sigma"][:, 1, 1].imag == 0.0)


def test_rpsh_energy_and_termination():
    # test/Dynamics/fssh.jl:210-233: RPSH on Tully 2 conserves the ring-polymer energy to rtol 1e-2
    n, nb = 32, 5
    rng = np.random.default_rng(1)
    r = np.full((n, nb), -10.0) + 0.1 * rng.standard_normal((n, nb))
    v = np.full((n, nb), 100 / 2000)
    o = O.run_rpsh(model=2, params=TULLY[2], mass=2000.0, r0=r, v0=v, nbeads=np.full(n, nb, np.int32), beta=100.0,
                   t0=0.0, t1=400.0, dt=0.1, seed=4)
    np.testing.assert_allclose(o["energy"][:, 1], o["energy"][:, 0], rtol=1e-2)
    # termination at |centroid| > 10
    o2 = O.run_rpsh(model=1, params=TULLY[1], mass=2000.0, r0=np.full((n, 8), -9.5), v0=np.full((n, 8), 0.01),
                    nbeads=np.full(n, 8, np.int32), beta=1024.0, t0=0.0, t1=20000.0, dt=1.0, seed=4, terminate_x=10.0)
    assert np.all(o2["nsteps"] < 20000)
    xc = o2["r"].mean(axis=1)
    assert np.all(np.abs(xc) > 10.0)


def test_rpsh_free_ring_polymer_centroid_moves_classically():
    # without a potential gradient (Tully 3 far left, constant diabats) the centroid drifts at constant velocity
    n, nb = 4, 8
    r0 = np.full((n, nb), -30.0) + np.linspace(-0.1, 0.1, nb)
    v0 = np.full((n, nb), 0.002)
    o = O.run_rpsh(model=3, params=TULLY[3], mass=2000.0, r0=r0, v0=v0, nbeads=np.full(n, nb, np.int32), beta=1024.0,
                   t0=0.0, t1=100.0, dt=1.0, seed=1)
    np.testing.assert_allclose(o["r"].mean(axis=1), -30.0 + 0.2, rtol=1e-9)


def test_mlp_oracle_gradient_finite_differences():
    # the surrogate network's reference gradient, without BF16 rounding, against central differences
    import mlp_oracle as MLP

    rng = np.random.default_rng(0)
    p = np.zeros(MLP.NP)
    p[0:64] = rng.uniform(-2, 2, 64)
    p[64:128] = rng.uniform(-2, 2, 64)
    p[128:4224] = rng.uniform(-0.2, 0.2, 4096)
    p[4224:4288] = rng.uniform(-0.1, 0.1, 64)
    p[4288:4352] = rng.uniform(-0.2, 0.2, 64)
    p[4352] = 0.3
    x = rng.uniform(-0.5, 0.5, 50)
    t = rng.uniform(0.0, 1.0, 50)
    _, g = MLP.loss_grad(p, x, t, 0.0, 2.0, rounding=False)
    for i in list(rng.choice(MLP.NP, 40, replace=False)) + [4352, 0, 64, 4224, 4288]:
        e = np.zeros(MLP.NP)
        e[i] = 1e-6
        lp, _ = MLP.loss_grad(p + e, x, t, 0.0, 2.0, rounding=False)
        lm, _ = MLP.loss_grad(p - e, x, t, 0.0, 2.0, rounding=False)
        assert abs((lp - lm) / 2e-6 - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), i


def test_mdef_oracle_friction_and_force_consistency():
    # force = dE/dx of the Fermi-weighted band energy (finite differences), friction >= 0,
    # Philox normals have unit variance
    import mdef_oracle as MO
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_mdef(4, M=40)
    model = MO.NewnsAnderson(k=wl["k"], g=wl["g"], delta=wl["delta"], V=1.0, eps=wl["eps"], weights=wl["V"] ** 2)
    x = np.linspace(-0.5, 0.5, 21)
    out = MO.electronic(model, x, wl["beta"], wl["sigma"])

    def energy(xx):
        w, _ = np.linalg.eigh(model.hamiltonian(xx))
        f = MO.fermi(w, 0.0, wl["beta"])
        return model.U0(xx) + np.sum(w * f, axis=1)

    h = 1e-6
    fd = (energy(x + h) - energy(x - h)) / (2 * h)
    # dE/dx = U0' + sum (d eps_i) (f_i + f'_i eps_i) at fixed mu: the reference force
    np.testing.assert_allclose(out["F"], fd, rtol=1e-5, atol=1e-8)
    assert np.all(out["friction"] >= -1e-15)
    z = MO.normal(7, np.arange(20000), 3)
    assert abs(z.mean()) < 0.03 and abs(z.std() - 1) < 0.03


# ---------------------------------------------------------------------------
# IESH oracle pins: the known answers of the reference's test/Dynamics/iesh.jl
# ---------------------------------------------------------------------------
def _iesh():
    import iesh_oracle as IO
    return IO


def test_iesh_unoccupied_known_answers():
    # test/Dynamics/iesh.jl:66-80 (1-based there): occupied 1:15 -> 16:31, occupied 6:20 -> 1:5, 21:31
    IO = _iesh()
    assert IO.unoccupied(list(range(15)), 31) == list(range(15, 31))
    assert IO.unoccupied(list(range(5, 20)), 31) == list(range(5)) + list(range(20, 31))


def test_iesh_overlap_and_akj_known_answers():
    # test/Dynamics/iesh.jl:87-109: overlap of the initial orbitals is the identity; with every
    # electron in state 1 only the first column is ones; A_kj(state, state) = 1
    IO = _iesh()
    n, ne = 31, 15
    psi = np.zeros((n, ne))
    psi[np.arange(ne), np.arange(ne)] = 1.0
    np.testing.assert_array_equal(IO.overlap(psi, list(range(ne))), np.eye(ne))
    S = IO.overlap(psi, [0] * ne)
    assert np.all(S[:, 0] == 1) and np.all(S[:, 1:] == 0)
    assert IO.akj(psi, list(range(ne)), 1.0, list(range(ne))) == pytest.approx(1.0)


def _narrow_band_model(IO, M=30):
    # the band of test/Dynamics/iesh.jl:17-25: Gamma = 6.4e-3, W = 3 Gamma, TrapezoidalRule(M, -W, W)
    G = 6.4e-3
    W = 3 * G
    eps = np.linspace(-W, W, M)
    V = np.full(M, np.sqrt(G / (2 * np.pi)) * np.sqrt(2 * W / (M - 1)))
    return IO.Metal3D(kxy=0.0, A=0.0, a=1.0, delta=0.0, B=0.0, b=1.0, eps=eps, V=V)


def test_iesh_fermi_dirac_zero_temperature_fills_lowest_states():
    # test/Dynamics/iesh.jl:39-44: at 0 K the sampled occupations are the lowest nelectrons states
    IO = _iesh()
    model = _narrow_band_model(IO)
    n = 16
    r = np.zeros((n, 3))
    w, _ = IO.eigen_continuous(model, r, np.tile(np.eye(31), (n, 1, 1)))
    st = IO.sample_fermi_dirac(w, 15, 1e12, 3, np.arange(n, dtype=np.uint64))
    np.testing.assert_array_equal(st, np.tile(np.arange(15), (n, 1)))


def test_iesh_fermi_dirac_statistics():
    # test/Dynamics/iesh.jl:44-64: sample averages of the occupations match the Fermi function
    # (isapprox on vectors: norm of the difference within 0.2 of the norm)
    IO = _iesh()
    model = _narrow_band_model(IO)
    n, ne, beta = 2000, 15, 1 / 9.5e-4
    r = np.zeros((n, 3))
    w, _ = IO.eigen_continuous(model, r, np.tile(np.eye(31), (n, 1, 1)))
    st = IO.sample_fermi_dirac(w, ne, beta, 7, np.arange(n, dtype=np.uint64))
    avg = np.zeros(31)
    for row in st:
        avg[row] += 1
    avg /= n
    lam = w[0]
    lo, hi = lam[0], lam[-1]
    for _ in range(200):  # Fermi level with sum f = ne (bisection)
        mu = 0.5 * (lo + hi)
        if np.sum(1 / (1 + np.exp(beta * (lam - mu)))) > ne:
            hi = mu
        else:
            lo = mu
    occ = 1 / (1 + np.exp(beta * (lam - mu)))
    assert np.linalg.norm(avg - occ) <= 0.2 * np.linalg.norm(occ)


def test_iesh_hop_rescaling_conserves_energy():
    # test/Dynamics/iesh.jl:122-152: after a successful hop dKE = -dE (rtol 1e-3)
    IO = _iesh()
    rng = np.random.default_rng(4)
    mass = np.array([2000.0, 2000.0, 2000.0])
    for _ in range(20):
        v = rng.normal(0, 0.01, 3)
        d = rng.normal(0, 1.0, 3)
        dE = rng.uniform(-0.01, 0.01)
        v2, ok = IO.rescale_velocity(v, d, mass, dE, 0)
        ke = lambda u: 0.5 * np.sum(mass * u * u)
        if ok:
            assert ke(v2) - ke(v) == pytest.approx(-dE, rel=1e-3, abs=1e-12)
        else:  # frustrated: velocity unchanged (:standard)
            np.testing.assert_array_equal(v2, v)


def test_iesh_dynamics_conserves_energy():
    # Verlet + exact propagator + rescaled hops: total energy (KE + U0 + occupied
    # eigenvalues) drifts only by the step error and the cached force after hops
    IO = _iesh()
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_iesh(4, nstates=20, nelectrons=10, z0=3.0)
    P = wl["params"]
    model = IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                       V=wl["V"])
    res = IO.run_iesh(model, mass=wl["mass"], ne=10, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"], dt=wl["dt"],
                      nsteps=300, seed=3)
    assert np.all(np.abs(res["energy"][:, 1] - res["energy"][:, 0]) < 5e-4)
    for t in range(4):  # orbitals stay orthonormal
        g = res["psi"][t].conj().T @ res["psi"][t]
        assert np.abs(g - np.eye(10)).max() < 1e-10


def _tully_vd(kind, x):
    import ctypes as C

    V, D, pp = np.zeros(3), np.zeros(3), np.zeros(8)
    pp[: len(TULLY[kind])] = TULLY[kind]
    dp = C.POINTER(C.c_double)
    O.lib().oracle_tully(kind, pp.ctypes.data_as(dp), C.c_double(x), V.ctypes.data_as(dp), D.ctypes.data_as(dp))
    return np.array([[V[0], V[1]], [V[1], V[2]]]), np.array([[D[0], D[1]], [D[1], D[2]]])


def _ehrenfest_dop853(kind, m, x0, v0, t1):
    """Independent high-accuracy Ehrenfest integration (the reference's test
    compares its integrator with Feagin12 the same way), in the diabatic basis:
    dc/dt = -i H(x) c, m dv/dt = -c^H dH/dx c, starting in the lower
    adiabatic state; returns x, v and the final adiabatic populations."""
    from scipy.integrate import solve_ivp

    c0 = np.linalg.eigh(_tully_vd(kind, x0)[0])[1][:, 0].astype(complex)

    def rhs(t, y):
        H, dH = _tully_vd(kind, y[0])
        c = y[2:4] + 1j * y[4:6]
        dc = -1j * (H @ c)
        return [y[1], -np.real(np.conj(c) @ dH @ c) / m, dc[0].real, dc[1].real, dc[0].imag, dc[1].imag]

    y0 = [x0, v0, c0[0].real, c0[1].real, c0[0].imag, c0[1].imag]
    y = solve_ivp(rhs, (0.0, t1), y0, method="DOP853", rtol=1e-12, atol=1e-13).y[:, -1]
    c = y[2:4] + 1j * y[4:6]
    Z = np.linalg.eigh(_tully_vd(kind, y[0])[0])[1]
    return y[0], y[1], np.abs(Z.T @ c) ** 2


def test_ehrenfest_reference_algorithm_comparison():
    """test/Dynamics/ehrenfest.jl:40-66: Tully model 2, mass 2000, p = 100
    from x = -10, t in [0, 50], dt = 2e-3 -- total energy conserved, and
    position, velocity and populations equal to an independent high-accuracy
    integration (the reference's tolerances: 1e-3 and 1e-1; met here to
    1e-6)."""
    pytest.importorskip("scipy")
    m, x0, v0 = 2000.0, -10.0, 100.0 / 2000.0
    res = O.run_fssh(model=2, params=TULLY[2], ndof=1, mass=m, r0=np.array([[x0]]), v0=np.array([[v0]]), t0=0.0,
                     t1=50.0, dt=2e-3, seed=1, ehrenfest=True, nthreads=1)
    assert res["sigma"][0, 0, 0].real == pytest.approx(np.abs(res["sigma"][0, 0, 0]))
    e0, e1 = res["energy"][0]
    assert abs(e1 - e0) < 1e-6
    xe, ve, pe = _ehrenfest_dop853(2, m, x0, v0, 50.0)
    assert res["r"][0, 0] == pytest.approx(xe, rel=1e-6)
    assert res["v"][0, 0] == pytest.approx(ve, rel=1e-6)
    assert res["sigma"][0, 0, 0].real == pytest.approx(pe[0], abs=1e-6)
    assert res["nhops"][0] == 0


@pytest.mark.parametrize("kind,p0,x0,t1", [(1, 20.0, -8.0, 1600.0), (2, 30.0, -8.0, 1100.0)])
def test_ehrenfest_through_the_coupling_region(kind, p0, x0, t1):
    """Ehrenfest (BAB + Tsit5 electronics, force from the step's initial
    density matrix, ehrenfest.jl:50-68) through the avoided crossing at
    dt = 0.1: second-order agreement with the high-accuracy integration."""
    pytest.importorskip("scipy")
    m = 2000.0
    res = O.run_fssh(model=kind, params=TULLY[kind], ndof=1, mass=m, r0=np.array([[x0]]), v0=np.array([[p0 / m]]),
                     t0=0.0, t1=t1, dt=0.1, seed=1, ehrenfest=True, nthreads=1)
    xe, ve, pe = _ehrenfest_dop853(kind, m, x0, p0 / m, t1)
    assert res["r"][0, 0] == pytest.approx(xe, rel=1e-4)
    assert res["v"][0, 0] == pytest.approx(ve, rel=1e-4)
    sig = res["sigma"][0]
    assert sig[0, 0].real == pytest.approx(pe[0], abs=1e-4)
    assert sig[1, 1].real == pytest.approx(pe[1], abs=1e-4)
    assert 0.2 < pe[1] < 0.8  # a genuine population transfer
    assert abs(res["energy"][0, 1] - res["energy"][0, 0]) < 1e-4 * res["energy"][0, 0]


def _metal_dop853_ehrenfest(model, mass, r0, v0, psi0, Z0, t1):
    """Exact Ehrenfest dynamics of the independent electrons in the diabatic
    basis (no eigenvectors, no couplings): d phi/dt = -i H phi,
    m dv/dt = -grad U0 - grad h sum_e |phi_0e|^2."""
    from scipy.integrate import solve_ivp

    N, ne = psi0.shape
    phi0 = Z0 @ psi0

    def rhs(t, y):
        r = y[0:3][None]
        phi = (y[6:6 + N * ne] + 1j * y[6 + N * ne:]).reshape(N, ne)
        imp = np.sum(np.abs(phi[0]) ** 2)
        dphi = -1j * (model.hamiltonian(r)[0] @ phi)
        return np.concatenate([y[3:6], -(model.grad_U0(r)[0] + model.grad_h(r)[0] * imp) / mass, dphi.real.ravel(),
                               dphi.imag.ravel()])

    y0 = np.concatenate([r0, v0, phi0.real.ravel(), phi0.imag.ravel()])
    y = solve_ivp(rhs, (0.0, t1), y0, method="DOP853", rtol=1e-10, atol=1e-12).y[:, -1]
    phi = (y[6:6 + N * ne] + 1j * y[6 + N * ne:]).reshape(N, ne)
    return y[0:3], y[3:6], np.sum(np.abs(phi[0]) ** 2)


def test_ehrenfest_na_fixed_step_against_high_accuracy():
    """test/Dynamics/ehrenfest_na.jl:22-49 restated on the three-dimensional
    metal model: the fixed-step integrator (VerletwithElectronics with the
    force of the pre-propagation orbitals) agrees with a high-accuracy
    integration of the same equations (the reference: Vern9 at 1e-15,
    rtol 1e-3 on positions and velocities), and its energy error is of first
    order in dt (the force lags the orbitals by one propagation)."""
    pytest.importorskip("scipy")
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "nqcdynamics.jl_gb300"))
    import iesh_oracle as IO
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_iesh(2, nstates=20, nelectrons=10, z0=3.5)
    P = wl["params"]
    model = IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                       V=wl["V"])
    t1 = 400 * wl["dt"]
    runs = {}
    for q in (2, 4):
        runs[q] = IO.run_iesh(model, mass=wl["mass"], ne=10, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"],
                              dt=wl["dt"] / q, nsteps=400 * q, seed=5, ehrenfest_na=True)
    res = runs[4]
    assert all(len(h) == 0 for h in res["hops"])
    for t in range(2):
        psi0 = np.zeros((20, 10))
        psi0[res["initial_state"][t], np.arange(10)] = 1.0
        Z0 = np.linalg.eigh(model.hamiltonian(wl["r0"][t:t + 1]))[1][0]
        r, v, imp = _metal_dop853_ehrenfest(model, wl["mass"], wl["r0"][t], wl["v0"][t], psi0, Z0, t1)
        np.testing.assert_allclose(res["r"][t], r, rtol=1e-3)
        np.testing.assert_allclose(res["v"][t], v, rtol=1e-3, atol=1e-6)
        assert abs(res["nimp"][t] - imp) < 5e-3
    d2 = np.abs(runs[2]["energy"][:, 1] - runs[2]["energy"][:, 0])
    d4 = np.abs(runs[4]["energy"][:, 1] - runs[4]["energy"][:, 0])
    assert np.all((d2 / d4 > 1.6) & (d2 / d4 < 2.5))


def test_decoherence_edc_reference_properties():
    """test/Dynamics/test_decoherence_corrections.jl: after one correction the
    unoccupied populations shrink, the occupied one grows, the norm stays 1;
    and each unoccupied coefficient is scaled by exp(-dt |E_j - E_s| / (1 + C/Ekin))
    (decoherence_corrections.jl:21-39, C = 0.1 by default)."""
    import iesh_oracle as IO

    rng = np.random.default_rng(3)
    psi = rng.random(4) + 1j * rng.random(4)
    psi /= np.linalg.norm(psi)
    orig = psi.copy()
    occupied, dt, E, ekin = 1, 0.1, np.array([0.1, 0.2, 0.3, 0.4]), 0.25
    IO.apply_decoherence_edc(psi, 0.1, occupied, dt, E, ekin)
    for i in range(4):
        if i != occupied:
            assert abs(psi[i]) ** 2 < abs(orig[i]) ** 2
            assert psi[i] == pytest.approx(orig[i] * np.exp(-dt * abs(E[i] - E[occupied]) / (1 + 0.1 / ekin)),
                                           rel=1e-14)
        else:
            assert abs(psi[i]) ** 2 > abs(orig[i]) ** 2
            assert np.angle(psi[i]) == pytest.approx(np.angle(orig[i]))
    assert np.linalg.norm(orig) == pytest.approx(1.0)
    assert np.linalg.norm(psi) == pytest.approx(1.0)


def test_rpmdef_oracle_reduces_to_baoab_for_one_bead():
    """BCOCB with one bead is BAOAB (the half Cayley steps of a free particle
    are half drifts), and the half step squares to the full Cayley step
    (ring_polymer.jl:71-82, half=true)."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "nqcdynamics.jl_gb300"))
    import mdef_oracle as MO
    from nqcd_gb300 import workload as WL

    for nb in (2, 4, 8):
        ch = MO.cayley_half(nb, 1024.0, 1.0)
        np.testing.assert_allclose(np.einsum("kij,kjl->kil", ch, ch), O.cayley(nb, 1024.0, 1.0), atol=1e-14)
    wl = WL.newns_anderson_mdef(3, M=40)
    model = MO.NewnsAnderson(k=wl["k"], g=wl["g"], delta=wl["delta"], V=1.0, eps=wl["eps"], weights=wl["V"] ** 2,
                             mu=wl["mu"])
    kw = dict(mass=wl["mass"], beta=wl["beta"], sigma=wl["sigma"], dt=wl["dt"], nsteps=50, seed=4)
    x1, v1 = MO.run_rpmdef(model, x0=wl["x0"][:, None], v0=wl["v0"][:, None], **kw)
    x2, v2 = MO.run_mdef(model, x0=wl["x0"], v0=wl["v0"], **kw)
    np.testing.assert_array_equal(x1[:, 0], x2)
    np.testing.assert_array_equal(v1[:, 0], v2)


def _rpiesh_case(n, nbeads, z0, **kw):
    IO = _iesh()
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_rpiesh(n, nbeads, z0=z0, **kw)
    P = wl["params"]
    model = IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                       V=wl["V"])
    return IO, wl, model


def test_rpiesh_spring_energy_known_answer():
    # get_spring_energy (ring_polymer.jl:85-107): m omega_n^2 / 2 times the sum of squared
    # neighbour distances around the ring; four beads on a unit square give 4
    IO = _iesh()
    r = np.array([[[0.0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]])
    beta, m = 8.0, 3.0
    assert IO.spring_energy(r, m, beta)[0] == pytest.approx(0.5 * m * (4 / beta) ** 2 * 4, rel=1e-15)
    r2 = np.array([[[0.0, 0, 0], [2, 0, 0]]])  # two beads: the pair counted once each way
    assert IO.spring_energy(r2, m, beta)[0] == pytest.approx(0.5 * m * (2 / beta) ** 2 * 8, rel=1e-15)


def test_rpiesh_oracle_one_bead_moves_the_nucleus_as_iesh():
    """With one bead the full Cayley step of the free ring polymer is the drift
    r + dt v, so BCBWavefunction moves the nucleus exactly as
    VerletwithElectronics; the orbitals differ only in the velocity used by the
    propagator (the step's start for BCBWavefunction, its end for
    VerletwithElectronics).  Far from the surface no hop happens."""
    IO, wl, model = _rpiesh_case(3, 1, 12.0, nstates=20, nelectrons=10)
    C = O.cayley(1, wl["beta"], wl["dt"])
    np.testing.assert_array_equal(C[0], [[1.0, wl["dt"]], [0.0, 1.0]])
    kw = dict(mass=wl["mass"], ne=10, beta=wl["beta"], dt=wl["dt"], nsteps=100, seed=2)
    a = IO.run_rpiesh(model, r0=wl["r0"], v0=wl["v0"], **kw)
    b = IO.run_iesh(model, r0=wl["r0"][:, 0, :], v0=wl["v0"][:, 0, :], **kw)
    assert all(len(h) == 0 for h in a["hops"]) and all(len(h) == 0 for h in b["hops"])
    np.testing.assert_array_equal(a["initial_state"], b["initial_state"])
    np.testing.assert_allclose(a["r"][:, 0, :], b["r"], rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(a["v"][:, 0, :], b["v"], rtol=1e-14, atol=1e-16)
    np.testing.assert_allclose(a["energy"], b["energy"], rtol=1e-13)
    np.testing.assert_allclose(a["psi"], b["psi"], atol=1e-6)


def test_rpiesh_oracle_conserves_ring_polymer_energy():
    # no hops far from the surface: kinetic + bead potentials + springs is conserved by the
    # symplectic BCB step to O(dt^2); orbitals stay orthonormal
    IO, wl, model = _rpiesh_case(3, 4, 12.0, nstates=16, nelectrons=8)
    res = IO.run_rpiesh(model, mass=wl["mass"], ne=8, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"], dt=wl["dt"],
                        nsteps=400, seed=5)
    assert all(len(h) == 0 for h in res["hops"])
    e0, e1 = res["energy"][:, 0], res["energy"][:, 1]
    assert np.all(np.abs(e1 - e0) < 1e-6 * np.abs(e0))
    for t in range(3):
        g = res["psi"][t].conj().T @ res["psi"][t]
        assert np.abs(g - np.eye(8)).max() < 1e-10


def test_rpiesh_workload_is_a_thermal_free_ring_polymer():
    """The ring-polymer IESH workload keeps every centroid at the classical
    workload's value and spreads the beads as the free ring polymer at
    beta_n = beta / nbeads: the mean spring energy per internal mode and
    Cartesian direction is 1 / (2 beta_n), and the bead velocities about the
    centroid have variance 1 / (beta_n m) times (nbeads - 1) / nbeads."""
    IO = _iesh()
    from nqcd_gb300 import workload as WL

    n, B = 4000, 8
    wl = WL.newns_anderson_rpiesh(n, B)
    base = WL.newns_anderson_iesh(n)
    np.testing.assert_allclose(wl["r0"].mean(1), base["r0"], atol=1e-12)
    np.testing.assert_allclose(wl["v0"].mean(1), base["v0"], atol=1e-15)
    bn, m = wl["beta"] / B, wl["mass"]
    spring = IO.spring_energy(wl["r0"], m, wl["beta"])  # m omega_n^2 / 2 sum |r_b - r_b+1|^2
    expect = 3 * (B - 1) / (2 * bn)
    assert spring.mean() == pytest.approx(expect, rel=0.02)
    dv = wl["v0"] - wl["v0"].mean(1, keepdims=True)
    assert dv.var() == pytest.approx((B - 1) / B / (bn * m), rel=0.02)


def test_tsit5_tableau_satisfies_the_order_five_conditions():
    """The Tsit5 tableau (Tsitouras, Comput. Math. Appl. 62, 770 (2011)), shared
    by the oracle and the kernels through csrc/nqcd_math.h, satisfies the row
    sums c_i = sum_j a_ij, the first-same-as-last property (the weights are the
    last row, c_6 = c_7 = 1) and all 17 Butcher order conditions up to order 5."""
    import re
    from pathlib import Path

    src = (Path(__file__).resolve().parent.parent / "nqcdynamics.jl_gb300" / "csrc" / "nqcd_math.h").read_text()
    body = src[src.index("struct Tsit5"):]
    body = body[: body.index("};")]
    val = {k: float(v) for k, v in re.findall(r"(\w+) = (-?[0-9.eE+-]+);", body)}
    A = np.zeros((7, 7))
    for (i, j) in [(i, j) for i in range(2, 8) for j in range(1, i)]:
        A[i - 1, j - 1] = val[f"a{i}{j}"]
    c = A.sum(axis=1)
    for i in range(2, 6):
        assert c[i - 1] == pytest.approx(val[f"c{i}"], abs=1e-15)
    assert c[5] == pytest.approx(1.0, abs=1e-14) and c[6] == pytest.approx(1.0, abs=1e-14)
    b = A[6]
    Ac, Ac2, Ac3 = A @ c, A @ c**2, A @ c**3
    AAc = A @ Ac
    conditions = [
        (b.sum(), 1.0), (b @ c, 1 / 2),
        (b @ c**2, 1 / 3), (b @ Ac, 1 / 6),
        (b @ c**3, 1 / 4), (b @ (c * Ac), 1 / 8), (b @ Ac2, 1 / 12), (b @ AAc, 1 / 24),
        (b @ c**4, 1 / 5), (b @ (c**2 * Ac), 1 / 10), (b @ (c * Ac2), 1 / 15), (b @ (c * AAc), 1 / 30),
        (b @ Ac**2, 1 / 20), (b @ Ac3, 1 / 20), (b @ (A @ (c * Ac)), 1 / 40), (b @ (A @ Ac2), 1 / 60),
        (b @ (A @ AAc), 1 / 120),
    ]
    for k, (got, want) in enumerate(conditions):
        assert got == pytest.approx(want, abs=5e-14), (k, got, want)


def test_iesh_force_is_the_gradient_of_the_adiabatic_energy():
    """Finite-difference consistency of the IESH acceleration (iesh.jl:190-207;
    rpiesh.jl:20-37 applies the same formula to each bead), as the reference
    checks acceleration!
    against FiniteDiff gradients (test/Dynamics/utils.jl:9-62): with
    dH = dh e0 e0^T the force -(grad U0 + grad h sum_occ z0_k^2) equals
    -grad(U0 + sum_occ l_k) at positions near the surface, for random
    occupied sets."""
    IO = _iesh()
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_iesh(1, nstates=24, nelectrons=12)
    P = wl["params"]
    model = IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                       V=wl["V"])
    rng = np.random.default_rng(11)

    def energy(r, occ):
        w = np.linalg.eigh(model.hamiltonian(r[None]))[0][0]
        return model.U0(r[None])[0] + w[occ].sum()

    for _ in range(8):
        r = np.array([rng.normal(0, 0.3), rng.normal(0, 0.3), rng.uniform(1.5, 4.0)])
        occ = np.sort(rng.choice(24, 12, replace=False))
        Z = np.linalg.eigh(model.hamiltonian(r[None]))[1][0]
        force = -(model.grad_U0(r[None])[0] + model.grad_h(r[None])[0] * np.sum(Z[0, occ] ** 2))
        h = 1e-5
        fd = np.array([-(energy(r + h * e, occ) - energy(r - h * e, occ)) / (2 * h) for e in np.eye(3)])
        np.testing.assert_allclose(force, fd, rtol=1e-6, atol=1e-10)


def _rpsh_continuous(r0, v0, *, mass, beta, dt, nsteps, seed, traj, substeps=2):
    """Independent integration of ring-polymer FSSH on Tully model 1: the
    continuous equations of motion! (rpsh.jl:12-28) integrated by RK4 with
    `substeps` sub-steps per dt, hop checks at the end of every step with the
    engine's Philox uniform (fewest_switches_probability!, fssh.jl:86-121,
    centroid velocity and coupling, SurfaceHoppingMethods.jl:81-103) and
    centroid momentum rescaling of every bead (surface_hopping.jl:64-99,
    rpsh.jl:30-50).  Beads feel -d/dx of their own eigenvalue of the occupied
    state and the springs omega_n^2 (2 x_j - x_j+1 - x_j-1), omega_n =
    nbeads / beta.  The adiabatic basis is the 2x2 rotation by
    theta = atan2(V12, V11) / 2, continuous because V12 > 0, with the lower
    state (sin theta, -cos theta): far left it is the identity, the oracle's
    starting gauge."""
    import iesh_oracle as IO

    A, Bp, C, D = TULLY[1]
    B = len(r0)
    wn2 = (B / beta) ** 2

    def model(x):
        e = np.exp(-Bp * np.abs(x))
        a = np.sign(x) * A * (1.0 - e)
        da = A * Bp * e
        c = C * np.exp(-D * x * x)
        dc = -2.0 * D * x * c
        return a, c, da, dc

    def centroid(x, v):
        a, c, da, dc = model(np.mean(x))
        rho = np.hypot(a, c)
        th = 0.5 * np.arctan2(c, a)
        z0 = np.array([np.sin(th), -np.cos(th)])
        z1 = np.array([np.cos(th), np.sin(th)])
        Dm = np.array([[da, dc], [dc, -da]])
        d01 = (z0 @ Dm @ z1) / (2.0 * rho)  # (Z^T dH Z)_01 / (w1 - w0)
        return np.array([-rho, rho]), d01, np.mean(v)

    def rhs(x, v, sig, s):
        a, c, da, dc = model(x)
        dw = (a * da + c * dc) / np.hypot(a, c)  # d/dx of the upper eigenvalue; the lower is -dw
        acc = (dw if s == 0 else -dw) / mass - wn2 * (2 * x - np.roll(x, 1) - np.roll(x, -1))
        w, d01, vc = centroid(x, v)
        Vm = np.array([[w[0], -1j * vc * d01], [1j * vc * d01, w[1]]])  # diag(w) - i v d, d10 = -d01
        return v, acc, -1j * (Vm @ sig - sig @ Vm)

    x, v = np.array(r0, float), np.array(v0, float)
    sig = np.array([[1.0, 0.0], [0.0, 0.0]], complex)
    s, hops = 0, []
    h = dt / substeps
    for step in range(1, nsteps + 1):
        for _ in range(substeps):
            k1 = rhs(x, v, sig, s)
            k2 = rhs(x + h / 2 * k1[0], v + h / 2 * k1[1], sig + h / 2 * k1[2], s)
            k3 = rhs(x + h / 2 * k2[0], v + h / 2 * k2[1], sig + h / 2 * k2[2], s)
            k4 = rhs(x + h * k3[0], v + h * k3[1], sig + h * k3[2], s)
            x = x + h / 6 * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0])
            v = v + h / 6 * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1])
            sig = sig + h / 6 * (k1[2] + 2 * k2[2] + 2 * k3[2] + k4[2])
        w, d01, vc = centroid(x, v)
        m = 1 - s
        dsm = d01 if s == 0 else -d01
        p = min(max(2.0 * vc * (sig[m, s] / sig[s, s]).real * dsm * dt, 0.0), 1.0)
        wh = IO.uniform(seed, np.array([traj], np.uint64), step, IO.RNG_HOP)
        u = IO.u53(wh[0], wh[1])[0]
        if u < p:
            d = -dsm  # d[new, old]
            aa, bb, cc = 0.5 * d * d / mass, d * vc, w[m] - w[s]
            disc = bb * bb - 4 * aa * cc
            if disc >= 0:
                root = np.sqrt(disc)
                gam = (bb + root) / (2 * aa) if bb < 0 else (bb - root) / (2 * aa)
                v = v - gam * d / mass
                hops.append((step, s, m))
                s = m
    return x, v, sig, s, hops


def test_rpsh_oracle_matches_a_continuous_integration():
    """The reference's BCBwithTsit5 test (test/Dynamics/bcbwithtsit5.jl:24-36):
    ring-polymer FSSH on Tully 1 with 10 beads at T = 1e-3, p = 20, beads at
    -5 + N(0, 1), the same random stream for both integrations, agreement to
    rtol 1e-3.  Here the oracle's BCBwithTsit5 restatement is compared with an
    independent fine-step integration of the continuous equations."""
    # the restated Tully 1 equals the oracle's model
    for xx in (-3.0, -0.4, 0.0, 0.7, 2.5):
        V, Dd = _tully_vd(1, xx)
        A, Bp, C, D = TULLY[1]
        e = np.exp(-Bp * abs(xx))
        np.testing.assert_allclose([V[0, 0], V[0, 1], Dd[0, 0], Dd[0, 1]],
                                   [np.sign(xx) * A * (1 - e), C * np.exp(-D * xx * xx), A * Bp * e,
                                    -2 * D * xx * C * np.exp(-D * xx * xx)], rtol=1e-12, atol=1e-15)
    B, n, mass, beta, dt, nsteps, seed = 10, 4, 2000.0, 1000.0, 0.1, 10000, 1
    rng = np.random.default_rng(1)
    r0 = -5.0 + rng.standard_normal((n, B))
    v0 = np.full((n, B), 20.0 / mass)
    o = O.run_rpsh(model=1, params=TULLY[1], mass=mass, r0=r0, v0=v0, nbeads=np.full(n, B, np.int32), beta=beta,
                   t0=0.0, t1=nsteps * dt, dt=dt, seed=seed)
    nhop = 0
    for t in range(n):
        x, v, sig, s, hops = _rpsh_continuous(r0[t], v0[t], mass=mass, beta=beta, dt=dt, nsteps=nsteps, seed=seed,
                                               traj=t)
        log = [tuple(h) for h in o["hop_log"][t] if h[0] >= 0]
        assert log == hops, (t, log, hops)
        nhop += len(hops)
        assert o["state"][t] == s
        np.testing.assert_allclose(o["r"][t], x, rtol=1e-3)
        np.testing.assert_allclose(o["v"][t], v, rtol=1e-3)
        np.testing.assert_allclose(o["sigma"][t], sig, atol=1e-3)
    assert nhop > 0  # the comparison covers hops


def test_mdef3d_oracle_reduces_to_one_dimension():
    """The 3-D MDEF restatement (friction tensor diagonalised as steps.jl:41-69
    does) with the atom on the z axis at rest in x, y follows the
    one-dimensional restatement of the same z-model: x and y stay 0, the
    tensor's only nonzero eigenvalue is along z, and z takes the noise of
    degree of freedom 2."""
    import iesh_oracle as IO
    import mdef_oracle as MO

    eps = np.linspace(-0.5, 0.5, 30)
    V = 0.04 * np.sqrt(eps[1] - eps[0]) * np.ones_like(eps)
    m3 = IO.Metal3D(kxy=2e-3, A=0.05, a=1.2, delta=0.05, B=0.3, b=0.8, eps=eps, V=V)

    class ZModel:
        mu = 0.0

        def dh(self, z):
            return m3.B * m3.b * np.exp(-m3.b * z)

        def dU0(self, z):
            return -m3.A * m3.a * np.exp(-m3.a * z)

        def hamiltonian(self, z):
            return m3.hamiltonian(np.stack([np.zeros_like(z), np.zeros_like(z), z], axis=1))

    n, mass, beta, sigma, dt = 6, 1837.0, 1000.0, 0.01, 20.0
    z0 = np.linspace(1.5, 3.5, n)
    vz0 = np.linspace(-3e-3, 1e-3, n)
    r0 = np.stack([np.zeros(n), np.zeros(n), z0], axis=1)
    v0 = np.stack([np.zeros(n), np.zeros(n), vz0], axis=1)
    r, v = MO.run_mdef3d(m3, mass=mass, mu=0.0, beta=beta, sigma=sigma, r0=r0, v0=v0, dt=dt, nsteps=40, seed=5)
    z, vz = MO.run_mdef(ZModel(), mass=mass, beta=beta, sigma=sigma, x0=z0, v0=vz0, dt=dt, nsteps=40, seed=5,
                        noise_dof=2)
    assert np.all(r[:, :2] == 0.0) and np.all(v[:, :2] == 0.0)
    np.testing.assert_allclose(r[:, 2], z, rtol=1e-12)
    np.testing.assert_allclose(v[:, 2], vz, rtol=1e-10, atol=1e-15)
    lam = MO.electronic3d(m3, r0, 0.0, beta, sigma)["friction"]
    assert np.all(lam[:, 2, 2] > 0) and np.all(lam[:, :2, :] == 0) and np.all(lam[:, :, :2] == 0)
