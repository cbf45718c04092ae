"""Generate the oracle fixtures at the benchmark configurations' own shapes.

    python tests/golden/make_config_shapes.py [name ...]

The MDEF and IESH oracles diagonalise dense matrices every step (numpy
LAPACK), which is too slow to run inside a GPU test at these shapes, so their
outputs are computed here once, over a spawn process pool in chunks of
trajectories (the random streams are keyed by global trajectory index, so the
chunking does not change a result), and committed:

  mdef_c4.npz    Newns-Anderson MDEF, 200 band states, 256 trajectories x
                 1000 steps of 0.1 fs (the benchmark system and step)
  rpmdef_c4.npz  ring-polymer MDEF on the same system, 4 beads,
                 32 trajectories x 1000 steps
  iesh_c5.npz    IESH, 80 states and 40 electrons, 64 trajectories x
                 1000 steps of 0.1 fs, started at z = 3 bohr where the
                 adsorbate level crosses the Fermi level, so hops occur

Each file holds the inputs (initial positions and velocities), the seed and
the oracle's outputs.  tests/test_gpu_config_shapes.py runs the plain FP64
GPU path on the same inputs and compares.
"""
from __future__ import annotations

import os
import sys
from concurrent.futures import ProcessPoolExecutor
from multiprocessing import get_context
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent

SEED = 20261203
NSTEPS = 1000


def _paths():
    sys.path.insert(0, str(ROOT / "oracle"))
    sys.path.insert(0, str(ROOT / "nqcdynamics.jl_gb300"))


def _mdef_model(wl):
    import mdef_oracle as MO

    return MO.NewnsAnderson(k=wl["k"], g=wl["g"], delta=wl["delta"], V=1.0, eps=wl["eps"], weights=wl["V"] ** 2,
                            mu=wl["mu"])


def _iesh_model(wl):
    import iesh_oracle as IO

    P = wl["params"]
    return IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                      V=wl["V"])


# ---------------------------------------------------------------- MDEF (C4)
MDEF_N, MDEF_M = 256, 200


def _mdef_chunk(lo, hi):
    _paths()
    import mdef_oracle as MO
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_mdef(MDEF_N, M=MDEF_M)
    x, v = MO.run_mdef(_mdef_model(wl), mass=wl["mass"], beta=wl["beta"], sigma=wl["sigma"], x0=wl["x0"][lo:hi],
                       v0=wl["v0"][lo:hi], dt=wl["dt"], nsteps=NSTEPS, seed=SEED, traj_offset=lo)
    return lo, x, v


def mdef_c4(pool):
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_mdef(MDEF_N, M=MDEF_M)
    x = np.zeros(MDEF_N)
    v = np.zeros(MDEF_N)
    for lo, xc, vc in pool.map(_mdef_chunk, range(0, MDEF_N, 16), range(16, MDEF_N + 16, 16)):
        x[lo:lo + len(xc)] = xc
        v[lo:lo + len(vc)] = vc
    return dict(x0=wl["x0"], v0=wl["v0"], seed=SEED, nsteps=NSTEPS, M=MDEF_M, x=x, v=v)


# ------------------------------------------------------ ring-polymer MDEF (C4)
RPMDEF_N, RPMDEF_B = 32, 4


def _rpmdef_inputs(wl):
    B = RPMDEF_B
    x0 = np.repeat(wl["x0"][:, None], B, axis=1) + 0.02 * np.sin(2 * np.pi * np.arange(B) / B)[None]
    v0 = np.repeat(wl["v0"][:, None], B, axis=1)
    return x0, v0


def _rpmdef_chunk(lo, hi):
    _paths()
    import mdef_oracle as MO
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_mdef(RPMDEF_N, M=MDEF_M)
    x0, v0 = _rpmdef_inputs(wl)
    x, v = MO.run_rpmdef(_mdef_model(wl), mass=wl["mass"], beta=wl["beta"], sigma=wl["sigma"], x0=x0[lo:hi],
                         v0=v0[lo:hi], dt=wl["dt"], nsteps=NSTEPS, seed=SEED, traj_offset=lo)
    return lo, x, v


def rpmdef_c4(pool):
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_mdef(RPMDEF_N, M=MDEF_M)
    x0, v0 = _rpmdef_inputs(wl)
    x = np.zeros_like(x0)
    v = np.zeros_like(v0)
    for lo, xc, vc in pool.map(_rpmdef_chunk, range(0, RPMDEF_N, 4), range(4, RPMDEF_N + 4, 4)):
        x[lo:lo + len(xc)] = xc
        v[lo:lo + len(vc)] = vc
    return dict(x0=x0, v0=v0, seed=SEED, nsteps=NSTEPS, M=MDEF_M, x=x, v=v)


# ---------------------------------------------------------------- IESH (C5)
IESH_N, IESH_NS, IESH_NE, IESH_Z0 = 64, 80, 40, 3.0
IESH_MAX_HOPS = 64
IESH_PSI_KEEP = 8  # full orbitals stored for the first trajectories


def _iesh_chunk(lo, hi):
    _paths()
    import iesh_oracle as IO
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_iesh(IESH_N, nstates=IESH_NS, nelectrons=IESH_NE, z0=IESH_Z0)
    o = IO.run_iesh(_iesh_model(wl), mass=wl["mass"], ne=IESH_NE, beta=wl["beta"], r0=wl["r0"][lo:hi],
                    v0=wl["v0"][lo:hi], dt=wl["dt"], nsteps=NSTEPS, seed=SEED, traj_offset=lo,
                    max_hops=IESH_MAX_HOPS)
    return lo, o


def iesh_c5(pool):
    from nqcd_gb300 import workload as WL

    wl = WL.newns_anderson_iesh(IESH_N, nstates=IESH_NS, nelectrons=IESH_NE, z0=IESH_Z0)
    n = IESH_N
    r = np.zeros((n, 3))
    v = np.zeros((n, 3))
    state = np.zeros((n, IESH_NE), np.int32)
    initial_state = np.zeros((n, IESH_NE), np.int32)
    nfrustrated = np.zeros(n, np.int32)
    energy = np.zeros((n, 2))
    hop_log = np.full((n, IESH_MAX_HOPS, 3), -1, np.int32)
    density = np.zeros((n, IESH_NS))
    psi = np.zeros((IESH_PSI_KEEP, IESH_NS, IESH_NE), np.complex128)
    for lo, o in pool.map(_iesh_chunk, range(0, n, 2), range(2, n + 2, 2)):
        hi = lo + o["r"].shape[0]
        r[lo:hi], v[lo:hi] = o["r"], o["v"]
        state[lo:hi], initial_state[lo:hi] = o["state"], o["initial_state"]
        nfrustrated[lo:hi], energy[lo:hi] = o["nfrustrated"], o["energy"]
        density[lo:hi] = np.sum(np.abs(o["psi"]) ** 2, axis=2)
        for t in range(lo, hi):
            hops = o["hops"][t - lo]
            assert len(hops) <= IESH_MAX_HOPS
            for k, h in enumerate(hops):
                hop_log[t, k] = h
            if t < IESH_PSI_KEEP:
                psi[t] = o["psi"][t - lo]
    return dict(r0=wl["r0"], v0=wl["v0"], seed=SEED, nsteps=NSTEPS, z0=IESH_Z0, r=r, v=v, state=state,
                initial_state=initial_state, nfrustrated=nfrustrated, energy=energy, hop_log=hop_log,
                density=density, psi_re=psi.real, psi_im=psi.imag)


CASES = {"mdef_c4": mdef_c4, "rpmdef_c4": rpmdef_c4, "iesh_c5": iesh_c5}


def main(names):
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"  # one BLAS thread per worker process
    _paths()
    with ProcessPoolExecutor(max_workers=os.cpu_count(), mp_context=get_context("spawn")) as pool:
        for name in names or CASES:
            np.savez_compressed(HERE / f"{name}.npz", **CASES[name](pool))
            print(name, (HERE / f"{name}.npz").stat().st_size, "bytes", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
