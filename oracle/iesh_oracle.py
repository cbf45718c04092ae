"""IESH oracle -- TEST INFRASTRUCTURE ONLY.

numpy FP64 restatement of NQCDynamics.jl's independent-electron surface
hopping on a Newns-Anderson (AndersonHolstein) metal:

  VerletwithElectronics.perform_step!   src/DynamicsMethods/IntegrationAlgorithms/verlet_with_electronics.jl:42-69
  propagate_wavefunction! /
  get_quantum_propagator                src/DynamicsUtils/wavefunction_dynamics.jl:15-58
  IESH acceleration!                    src/DynamicsMethods/SurfaceHoppingMethods/iesh.jl:190-207
  evaluate_hopping_probability!         iesh.jl:231-283 (with the estimate screen :251-254)
  evaluate_v_dot_d!, calculate_Akj,
  compute_overlap!                      iesh.jl:285-316
  select_new_state                      iesh.jl:318-335
  iesh_check_hop! / iesh_execute_hop!   iesh.jl:390-407
  rescale_velocity!                     surface_hopping.jl:64-99
  sample_fermi_dirac_distribution       src/DynamicsUtils/DynamicsUtils.jl:194-208
  set_unoccupied_states!                DynamicsUtils.jl:162-171

Electronic structure as the reference's cache computes it: dense
eigen-decomposition (LAPACK) with eigenvector signs fixed by continuity with
the previous step (identity first), Z^T dH Z, couplings A_ij / (l_j - l_i).
The propagator is the exact U exp(-i mu dt) U^H of the effective
Hamiltonian (LAPACK eigh of the Hermitian matrix), determinants by LU.

Random numbers: the engine's Philox4x32-10 stream; one 53-bit uniform per
trajectory and step for the hop test (stream HOP), three per Metropolis
iteration of the initial occupations (stream FERMI_DIRAC).

Model (AndersonHolstein with a 3-D impurity): one atom, coordinates
(x, y, z); U0 = k_xy (x^2 + y^2)/2 + A exp(-a z);
h = U1 - U0 = delta - B exp(-b z); constant couplings V_k; bath levels e_k.
"""
from __future__ import annotations

import numpy as np

from mdef_oracle import philox

RNG_HOP = 1
RNG_INIT_FD = 4


def u53(w0, w1):
    a = ((np.asarray(w0).astype(np.uint64) << np.uint64(32)) | np.asarray(w1).astype(np.uint64)) >> np.uint64(11)
    return a.astype(np.float64) * 2.0**-53


def uniform(seed, traj, step, stream):
    traj = np.asarray(traj, dtype=np.uint64)
    w = philox((traj & np.uint64(0xFFFFFFFF)).astype(np.uint32), (traj >> np.uint64(32)).astype(np.uint32),
               np.full(traj.shape, step, np.uint32), np.full(traj.shape, stream, np.uint32), seed & 0xFFFFFFFF,
               (seed >> 32) & 0xFFFFFFFF)
    return w


class Metal3D:
    def __init__(self, *, kxy, A, a, delta, B, b, eps, V):
        self.kxy, self.A, self.a, self.delta, self.B, self.b = kxy, A, a, delta, B, b
        self.eps = np.asarray(eps, np.float64)
        self.V = np.asarray(V, np.float64)
        self.nstates = 1 + len(self.eps)

    def h(self, r):
        return self.delta - self.B * np.exp(-self.b * r[..., 2])

    def grad_h(self, r):
        g = np.zeros_like(r)
        g[..., 2] = self.B * self.b * np.exp(-self.b * r[..., 2])
        return g

    def grad_U0(self, r):
        g = np.zeros_like(r)
        g[..., 0] = self.kxy * r[..., 0]
        g[..., 1] = self.kxy * r[..., 1]
        g[..., 2] = -self.A * self.a * np.exp(-self.a * r[..., 2])
        return g

    def U0(self, r):
        return 0.5 * self.kxy * (r[..., 0] ** 2 + r[..., 1] ** 2) + self.A * np.exp(-self.a * r[..., 2])

    def hamiltonian(self, r):
        n = r.shape[0]
        N = self.nstates
        H = np.zeros((n, N, N))
        H[:, 0, 0] = self.h(r)
        H[:, 0, 1:] = self.V
        H[:, 1:, 0] = self.V
        idx = np.arange(1, N)
        H[:, idx, idx] = self.eps
        return H


def eigen_continuous(model, r, Zprev):
    w, Z = np.linalg.eigh(model.hamiltonian(r))
    sgn = np.where(np.einsum("tki,tki->ti", Z, Zprev) < 0, -1.0, 1.0)
    return w, Z * sgn[:, None, :]


def unoccupied(state, nstates):
    """Ascending unoccupied states (set_unoccupied_states!, DynamicsUtils.jl:162-171)."""
    occ = set(int(x) for x in state)
    return [s for s in range(nstates) if s not in occ]


def overlap(psi, state):
    """S[j, i] = psi[state[j], i] (compute_overlap!, iesh.jl:309-316)."""
    return psi[np.asarray(state), :]


def akj(psi, state, det_s, new_state):
    """det S conj(det S') (calculate_Akj, iesh.jl:301-306)."""
    return det_s * np.conj(np.linalg.det(overlap(psi, new_state)))


def rescale_velocity(v, d, mass, dE, rescaling):
    """Momentum rescaling along d for a hop with potential-energy change dE
    (rescale_velocity!, surface_hopping.jl:64-168): returns (v, accepted)."""
    aa = np.sum(d * d / mass) / 2
    bb = np.dot(d, v)
    disc = bb * bb - 4 * aa * dE
    if disc < 0:
        if rescaling == 1:  # :vinversion
            dn = d / np.linalg.norm(d)
            v = v - 2 * np.dot(v, dn) * dn
        return v, False
    root = np.sqrt(disc)
    gam = (bb + root) / (2 * aa) if bb < 0 else (bb - root) / (2 * aa)
    return v - gam * d / mass, True


def sample_fermi_dirac(energies, ne, beta, seed, traj_ids):
    """Metropolis occupations: Ne electrons in N states (DynamicsUtils.jl:194-208)."""
    n, N = energies.shape
    states = np.tile(np.arange(ne), (n, 1))
    for it in range(N * ne):
        wa = uniform(seed, traj_ids, it, RNG_INIT_FD)
        wb = uniform(seed, traj_ids, it, RNG_INIT_FD + 16)
        ua, ub, uc = u53(wa[0], wa[1]), u53(wa[2], wa[3]), u53(wb[0], wb[1])
        for t in range(n):
            ci = min(int(ua[t] * ne), ne - 1)
            occ = set(states[t].tolist())
            unocc = [s for s in range(N) if s not in occ]
            j = unocc[min(int(ub[t] * len(unocc)), len(unocc) - 1)]
            i = states[t, ci]
            prob = np.exp(-beta * (energies[t, j] - energies[t, i]))
            if prob > uc[t]:
                states[t, ci] = j
    return np.sort(states, axis=1)


def total_energy(model, r, v, w, state, mass):
    """KE + U0 + sum of occupied eigenvalues (iesh.jl:380-388)."""
    return 0.5 * mass * np.sum(v * v, axis=1) + model.U0(r) + np.take_along_axis(w, state, axis=1).sum(1)


def total_energy_ehrenfest_na(model, r, v, w, psi, mass):
    """KE + U0 + sum_e sum_i E_i |psi_ie|^2 (ehrenfest_na.jl:106-117)."""
    return 0.5 * mass * np.sum(v * v, axis=1) + model.U0(r) + np.einsum("ti,tie->t", w, np.abs(psi) ** 2)


def impurity_population_ehrenfest_na(psi, Z):
    """Impurity population of the orbitals: sum_e |sum_a z0_a psi_ae|^2."""
    amp = np.einsum("ta,tae->te", Z[:, 0, :], psi)
    return (np.abs(amp) ** 2).sum(1)


def impurity_population(psi, Z, state):
    """Row 0 of iesh_diabatic_population (iesh.jl:351-369) per trajectory."""
    z0 = Z[:, 0, :]
    amp = np.einsum("ta,tan->tn", z0, psi)
    sq = np.einsum("ta,tan->tn", z0 * z0, np.abs(psi) ** 2)
    return (np.abs(amp) ** 2 - sq).sum(1) + (np.take_along_axis(z0, state, axis=1) ** 2).sum(1)


def apply_decoherence_edc(psi, C, occupied, dt, E, ekin):
    """apply_decoherence_correction! (decoherence_corrections.jl:21-39): Eq. 17
    of Granucci and Persico, J. Chem. Phys. 126, 134114 (2007), in place."""
    norm = 0.0
    for i in range(len(psi)):
        if i != occupied:
            tau = (1.0 + C / ekin) / abs(E[i] - E[occupied])
            psi[i] = psi[i] * np.exp(-dt / tau)
            norm += abs(psi[i]) ** 2
    cm = psi[occupied]
    psi[occupied] = cm * np.sqrt((1.0 - norm) / abs(cm) ** 2)


def run_iesh(model, *, mass, ne, beta, r0, v0, dt, nsteps, seed, traj_offset=0, rescaling=0, max_hops=16,
             estimate=True, initial_state=None, ehrenfest_na=False, decoherence_C=0.0, h_last=None):
    """estimate: the reference's estimate_probability screen (iesh.jl:251-254).
    initial_state: given occupations (ntraj, ne) instead of Fermi-Dirac sampling.
    ehrenfest_na: Simulation{EhrenfestNA} instead (ehrenfest_na.jl): the same
    integrator and initial orbitals (verlet_with_electronics.jl:51-65), the
    force of the orbitals before propagation, -sum_e sum_nm A_nm
    Re(psi_ne conj(psi_me)) = -dh |sum_n z0_n psi_ne|^2 summed over e
    (ehrenfest_na.jl:74-90; A = dh z0 z0^T for this model), and no hops.
    decoherence_C > 0: DecoherenceCorrectionEDC(C) applied to every electron's
    column after each step's hop (iesh.jl:424-441).
    h_last: length of the last step when the time span is not a whole number
    of steps.  The integrator takes the shortened step (Verlet and propagator,
    verlet_with_electronics.jl:42-69 read integrator.dt); the hop probability
    and the decoherence correction read get_proposed_dt, the full dt
    (iesh.jl:390-398, 430-441)."""
    n = r0.shape[0]
    N = model.nstates
    traj = np.arange(n, dtype=np.uint64) + np.uint64(traj_offset)
    r = np.asarray(r0, np.float64).copy()
    v = np.asarray(v0, np.float64).copy()
    Z = np.tile(np.eye(N), (n, 1, 1))
    w, Z = eigen_continuous(model, r, Z)
    states = sample_fermi_dirac(w, ne, beta, seed, traj) if initial_state is None else np.array(initial_state)
    psi = np.zeros((n, N, ne), np.complex128)
    for t in range(n):
        psi[t, states[t], np.arange(ne)] = 1.0
    state = states.copy()
    hops = [[] for _ in range(n)]
    nfr = np.zeros(n, np.int32)

    def accel(w, Z, r, state, psi):
        gh = model.grad_h(r)
        z0 = Z[:, 0, :]
        if ehrenfest_na:
            occsum = (np.abs(np.einsum("ta,tae->te", z0, psi)) ** 2).sum(1)
        else:
            occsum = (np.take_along_axis(z0, state, axis=1) ** 2).sum(1)
        return -(model.grad_U0(r) + gh * occsum[:, None]) / mass

    def energy(w, psi):
        if ehrenfest_na:
            return total_energy_ehrenfest_na(model, r, v, w, psi, mass)
        return total_energy(model, r, v, w, state, mass)

    k = accel(w, Z, r, state, psi)
    e0 = energy(w, psi)
    nfull = 0
    for step in range(1, nsteps + 1):
        hs = h_last if (h_last is not None and step == nsteps) else dt  # this step's length
        vt = v + (hs / 2) * k
        r = r + hs * vt
        w, Z = eigen_continuous(model, r, Z)
        k = accel(w, Z, r, state, psi)
        v = vt + (hs / 2) * k
        gh = model.grad_h(r)
        z0 = Z[:, 0, :]
        lam_diff = w[:, None, :] - w[:, :, None]  # l_j - l_i
        with np.errstate(divide="ignore", invalid="ignore"):
            base = z0[:, :, None] * z0[:, None, :] / lam_diff
        idx = np.arange(N)
        base[:, idx, idx] = 0.0
        vdh = np.einsum("ta,ta->t", v, gh)  # sum_alpha v_alpha dh/dq_alpha
        vd = vdh[:, None, None] * base  # sum_alpha v_alpha d_alpha
        Heff = np.zeros((n, N, N), np.complex128)
        Heff[:, idx, idx] = w
        Heff -= 1j * vd
        mu, U = np.linalg.eigh(Heff)
        P = np.einsum("tij,tj,tkj->tik", U, np.exp(-1j * mu * hs), U.conj())
        psi = P @ psi
        if ehrenfest_na:
            continue
        # hopping
        wh = uniform(seed, traj, step, RNG_HOP)
        rnd = u53(wh[0], wh[1])
        for t in range(n):
            st = state[t]
            unocc = np.array([s for s in range(N) if s not in set(st.tolist())])
            S = psi[t][st, :]
            detS = np.linalg.det(S)
            Akk = abs(detS) ** 2
            pref = 2 * dt / Akk
            vdd = np.zeros((N, ne))
            for nn in range(ne):
                vdd[unocc, nn] -= vd[t][unocc, st[nn]]
            est = pref * np.abs(vdd).sum() * (abs(detS.real) + abs(detS.imag))
            if estimate and est < rnd[t]:
                continue
            nfull += 1
            prob = np.zeros((N, ne))
            for nn in range(ne):
                for m in unocc:
                    s2 = st.copy()
                    s2[nn] = m
                    det2 = np.linalg.det(psi[t][s2, :])
                    prob[m, nn] = pref * (detS * np.conj(det2)).real * vdd[m, nn]
            prob = np.clip(prob, 0, 1)
            cum = 0.0
            new = None
            for nn in range(ne):
                for m in unocc:
                    cum += prob[m, nn]
                    if rnd[t] < cum:
                        new = (nn, m)
                        break
                if new:
                    break
            if new is None:
                continue
            nn, m = new
            old = st[nn]
            accept = True
            if rescaling != 2:
                d = gh[t] * z0[t, m] * z0[t, old] / (w[t, old] - w[t, m])  # d_alpha[m, old]
                v[t], accept = rescale_velocity(v[t], d, mass, w[t, m] - w[t, old], rescaling)
            if accept:
                state[t, nn] = m
                hops[t].append((step, int(old), int(m)))
            else:
                nfr[t] += 1
        if decoherence_C > 0.0:
            for t in range(n):
                ekin = 0.5 * mass * np.sum(v[t] * v[t])
                for e in range(ne):
                    apply_decoherence_edc(psi[t, :, e], decoherence_C, int(state[t, e]), dt, w[t], ekin)
    e1 = energy(w, psi)
    nimp = impurity_population_ehrenfest_na(psi, Z) if ehrenfest_na else impurity_population(psi, Z, state)
    return dict(r=r, v=v, psi=psi, state=state, hops=hops, nfrustrated=nfr, Z=Z, w=w, initial_state=states,
                energy=np.stack([e0, e1], axis=1), nimp=nimp, nfull=nfull)


def spring_energy(r, mass, beta):
    """get_spring_energy (ring_polymer.jl:85-107): m omega_n^2 / 2 sum over
    neighbouring beads (cyclic) of |r_b - r_b+1|^2, omega_n = nbeads / beta."""
    B = r.shape[1]
    wn = B / beta
    d = r - np.roll(r, -1, axis=1)
    return 0.5 * mass * wn * wn * np.sum(d * d, axis=(1, 2))


def run_rpiesh(model, *, mass, ne, beta, r0, v0, dt, nsteps, seed, traj_offset=0, rescaling=0, estimate=True,
               initial_state=None, save_stride=0):
    """RingPolymerSimulation{AdiabaticIESH} (rpiesh.jl) with BCBWavefunction
    (bcb_wavefunction.jl:37-69).  r0, v0: (ntraj, nbeads, 3).

    Step: v' = v + dt/2 k; full Cayley step of the free ring polymer in
    normal modes (cayley_propagator(half=false), ring_polymer.jl:71-82,
    omega_n = nbeads / beta); bead forces from each bead's own eigenstates
    summed over the shared occupied set (rpiesh.jl:20-37); v = v' + dt/2 k;
    orbitals propagated with the centroid velocity of the step's START and the
    centroid eigenvalues and couplings of the step's END (the calculator
    cache holds the end positions when propagate_wavefunction! reads it,
    bcb_wavefunction.jl:59-68, SurfaceHoppingMethods.jl:81-103).  Hops use
    the final centroid velocity and couplings (iesh.jl:231-298); an accepted
    hop shifts every bead's velocity by the same -gamma d / m and a frustrated
    :vinversion hop inverts the centroid velocity along d in every bead
    (rpsh.jl:30-50).  Fermi-Dirac occupations come from the centroid
    eigenvalues (iesh.jl:99-128).  Energy: kinetic + sum over beads of
    U0 + occupied eigenvalues (rpiesh.jl:39-52) + spring energy.
    save_stride > 0: observables at step 0 and every save_stride steps, after
    the step's hops, per trajectory (nsave, ntraj, 4): centroid height z,
    kinetic energy of all beads (classical_kinetic_energy,
    DynamicsUtils.jl:122-132), impurity population of the centroid
    eigenstates (iesh.jl:351-369), and the potential of
    classical_potential_energy (rpiesh.jl:40-52: sum over beads of U0 and
    the occupied eigenvalues, no spring term)."""
    import oracle as O

    n, B, _ = r0.shape
    N = model.nstates
    traj = np.arange(n, dtype=np.uint64) + np.uint64(traj_offset)
    r = np.asarray(r0, np.float64).copy()
    v = np.asarray(v0, np.float64).copy()
    U = O.nm_transform(B)  # U[j, k]: bead j, mode k
    C = O.cayley(B, beta, dt)

    def free(r, v):
        q = np.einsum("tbd,bk->tkd", r, U)
        p = np.einsum("tbd,bk->tkd", v, U)
        q2 = C[None, :, 0, 0, None] * q + C[None, :, 0, 1, None] * p
        p2 = C[None, :, 1, 0, None] * q + C[None, :, 1, 1, None] * p
        return np.einsum("tkd,bk->tbd", q2, U), np.einsum("tkd,bk->tbd", p2, U)

    def beads(r):
        w, Z = np.linalg.eigh(model.hamiltonian(r.reshape(n * B, 3)))
        return w.reshape(n, B, N), (Z[:, 0, :] ** 2).reshape(n, B, N)

    def accel(r, state):
        _, z2 = beads(r)
        occsum = np.take_along_axis(z2, np.repeat(state[:, None, :], B, axis=1), axis=2).sum(2)
        gh = model.grad_h(r.reshape(n * B, 3)).reshape(n, B, 3)
        gu = model.grad_U0(r.reshape(n * B, 3)).reshape(n, B, 3)
        return -(gu + gh * occsum[:, :, None]) / mass

    def energy(r, v, state):
        w, _ = beads(r)
        band = np.take_along_axis(w, np.repeat(state[:, None, :], B, axis=1), axis=2).sum(2)
        pot = (model.U0(r.reshape(n * B, 3)).reshape(n, B) + band).sum(1)
        return 0.5 * mass * np.sum(v * v, axis=(1, 2)) + pot + spring_energy(r, mass, beta)

    Zc = np.tile(np.eye(N), (n, 1, 1))
    wc, Zc = eigen_continuous(model, r.mean(1), Zc)
    states = sample_fermi_dirac(wc, ne, beta, seed, traj) if initial_state is None else np.array(initial_state)
    psi = np.zeros((n, N, ne), np.complex128)
    for t in range(n):
        psi[t, states[t], np.arange(ne)] = 1.0
    state = states.copy()
    hops = [[] for _ in range(n)]
    nfr = np.zeros(n, np.int32)
    k = accel(r, state)
    e0 = energy(r, v, state)
    idx = np.arange(N)
    obs = []

    def observe(Zc):
        w, _ = beads(r)
        band = np.take_along_axis(w, np.repeat(state[:, None, :], B, axis=1), axis=2).sum(2)
        pot = (model.U0(r.reshape(n * B, 3)).reshape(n, B) + band).sum(1)
        ke = 0.5 * mass * np.sum(v * v, axis=(1, 2))
        obs.append(np.stack([r.mean(1)[:, 2], ke, impurity_population(psi, Zc, state), pot], axis=1))

    if save_stride:
        observe(Zc)
    for step in range(1, nsteps + 1):
        vc_prev = v.mean(1)
        vt = v + (dt / 2) * k
        r, vt = free(r, vt)
        k = accel(r, state)
        v = vt + (dt / 2) * k
        rc = r.mean(1)
        wc, Zc = eigen_continuous(model, rc, Zc)
        gh = model.grad_h(rc)
        z0 = Zc[:, 0, :]
        with np.errstate(divide="ignore", invalid="ignore"):
            base = z0[:, :, None] * z0[:, None, :] / (wc[:, None, :] - wc[:, :, None])
        base[:, idx, idx] = 0.0
        Heff = np.zeros((n, N, N), np.complex128)
        Heff[:, idx, idx] = wc
        Heff -= 1j * np.einsum("ta,ta->t", vc_prev, gh)[:, None, None] * base
        mu, Uh = np.linalg.eigh(Heff)
        psi = np.einsum("tij,tj,tkj->tik", Uh, np.exp(-1j * mu * dt), Uh.conj()) @ psi
        vc = v.mean(1)
        vd = np.einsum("ta,ta->t", vc, gh)[:, None, None] * base
        wh = uniform(seed, traj, step, RNG_HOP)
        rnd = u53(wh[0], wh[1])
        for t in range(n):
            st = state[t]
            unocc = np.array([s for s in range(N) if s not in set(st.tolist())])
            detS = np.linalg.det(psi[t][st, :])
            pref = 2 * dt / abs(detS) ** 2
            vdd = np.zeros((N, ne))
            for nn in range(ne):
                vdd[unocc, nn] -= vd[t][unocc, st[nn]]
            if estimate and pref * np.abs(vdd).sum() * (abs(detS.real) + abs(detS.imag)) < rnd[t]:
                continue
            prob = np.zeros((N, ne))
            for nn in range(ne):
                for m in unocc:
                    s2 = st.copy()
                    s2[nn] = m
                    prob[m, nn] = pref * (detS * np.conj(np.linalg.det(psi[t][s2, :]))).real * vdd[m, nn]
            prob = np.clip(prob, 0, 1)
            cum, new = 0.0, None
            for nn in range(ne):
                for m in unocc:
                    cum += prob[m, nn]
                    if rnd[t] < cum:
                        new = (nn, m)
                        break
                if new:
                    break
            if new is None:
                continue
            nn, m = new
            old = st[nn]
            accept = True
            if rescaling != 2:
                d = gh[t] * z0[t, m] * z0[t, old] / (wc[t, old] - wc[t, m])
                vc_new, accept = rescale_velocity(vc[t], d, mass, wc[t, m] - wc[t, old], rescaling)
                v[t] += (vc_new - vc[t])[None, :]  # the same shift in every bead
            if accept:
                state[t, nn] = m
                hops[t].append((step, int(old), int(m)))
            else:
                nfr[t] += 1
        if save_stride and step % save_stride == 0:
            observe(Zc)
    e1 = energy(r, v, state)
    return dict(r=r, v=v, psi=psi, state=state, hops=hops, nfrustrated=nfr, initial_state=states,
                energy=np.stack([e0, e1], axis=1), obs=np.array(obs) if save_stride else None)
