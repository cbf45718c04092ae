"""Generate the golden fixtures of this directory from the oracle.

    python tests/golden/make_golden.py

Each .npz holds the inputs and the oracle's outputs of one small case per
method; tests/test_golden.py checks that the oracle still reproduces them
(CPU) and tests/test_gpu_golden.py that the GPU kernels match them.  The
oracle follows the reference's algorithms (oracle/*), whose own test vectors
pin it (tests/test_oracle_pins.py).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "nqcdynamics.jl_gb300"))

SEED = 20261203
TULLY1 = (0.01, 1.6, 0.005, 1.0)


def fssh_tully1():
    import oracle as O

    rng = np.random.default_rng(1)
    n = 32
    r0 = np.full((n, 1), -10.0)
    v0 = rng.uniform(8.0, 30.0, (n, 1)) / 2000.0
    res = O.run_fssh(model=1, params=TULLY1, ndof=1, mass=2000.0, r0=r0, v0=v0, t0=0.0, t1=1500.0, dt=1.0, seed=SEED,
                     rescaling=0, max_hops=16)
    return dict(r0=r0, v0=v0, r=res["r"], v=res["v"], sigma_re=res["sigma"].real, sigma_im=res["sigma"].imag,
                state=res["state"], nhops=res["nhops"], hop_log=res["hop_log"])


def fssh_spinboson():
    import oracle as O
    from nqcd_gb300 import workload as WL

    n, modes = 8, 20
    w, c, r0, v0 = WL.spin_boson_inputs(n, modes)
    res = O.run_fssh(model=10, params=(0.0, 1.0), ndof=modes, mass=1.0, r0=r0, v0=v0, t0=0.0, t1=5.0, dt=0.05,
                     seed=SEED, init_kind=2, init_state=0, bath_c=c, bath_w2=w * w, max_hops=16)
    return dict(w=w, c=c, r0=r0, v0=v0, r=res["r"], v=res["v"], sigma_re=res["sigma"].real,
                sigma_im=res["sigma"].imag, state=res["state"], nhops=res["nhops"], hop_log=res["hop_log"])


def rpsh_mixed():
    import oracle as O

    rng = np.random.default_rng(2)
    n, bmax = 24, 16
    nb = rng.choice(np.array([4, 8, 16], np.int32), n).astype(np.int32)
    r0 = np.full((n, bmax), -9.5) + 0.05 * rng.standard_normal((n, bmax))
    v0 = np.repeat(rng.uniform(8.0, 30.0, (n, 1)) / 2000.0, bmax, axis=1)
    res = O.run_rpsh(model=1, params=TULLY1, mass=2000.0, r0=r0, v0=v0, nbeads=nb, beta=1024.0, t0=0.0, t1=800.0,
                     dt=1.0, seed=SEED, rescaling=0, terminate_x=10.0, max_hops=16)
    return dict(r0=r0, v0=v0, nbeads=nb, r=res["r"], v=res["v"], state=res["state"], nsteps=res["nsteps"],
                hop_log=res["hop_log"], energy=res["energy"])


def mdef_small():
    import mdef_oracle as MO
    from nqcd_gb300 import workload as WL

    n = 8
    wl = WL.newns_anderson_mdef(n, M=40)
    model = MO.NewnsAnderson(k=wl["k"], g=wl["g"], delta=wl["delta"], V=1.0, eps=wl["eps"], weights=wl["V"] ** 2,
                             mu=wl["mu"])
    x, v = MO.run_mdef(model, mass=wl["mass"], beta=wl["beta"], sigma=wl["sigma"], x0=wl["x0"], v0=wl["v0"],
                       dt=wl["dt"], nsteps=100, seed=SEED)
    return dict(x0=wl["x0"], v0=wl["v0"], eps=wl["eps"], V=wl["V"],
                params=np.array([wl["k"], wl["g"], wl["delta"], wl["mu"], wl["sigma"], wl["mass"], wl["beta"],
                                 wl["dt"]]), x=x, v=v)


def iesh_small():
    import iesh_oracle as IO
    from nqcd_gb300 import workload as WL

    n = 4
    wl = WL.newns_anderson_iesh(n, nstates=20, nelectrons=10, z0=3.5)
    P = wl["params"]
    model = IO.Metal3D(kxy=P["kxy"], A=P["A"], a=P["a"], delta=P["delta"], B=P["B"], b=P["b"], eps=wl["eps"],
                       V=wl["V"])
    res = IO.run_iesh(model, mass=wl["mass"], ne=10, beta=wl["beta"], r0=wl["r0"], v0=wl["v0"], dt=wl["dt"],
                      nsteps=200, seed=SEED)
    hops = np.full((n, 16, 3), -1, np.int32)
    for t in range(n):
        for k, h in enumerate(res["hops"][t][:16]):
            hops[t, k] = h
    return dict(r0=wl["r0"], v0=wl["v0"], r=res["r"], v=res["v"], psi_re=res["psi"].real, psi_im=res["psi"].imag,
                state=res["state"], initial_state=res["initial_state"], hop_log=hops, energy=res["energy"])


CASES = {"fssh_tully1": fssh_tully1, "fssh_spinboson": fssh_spinboson, "rpsh_mixed": rpsh_mixed,
         "mdef_small": mdef_small, "iesh_small": iesh_small}


def main():
    for name, fn in CASES.items():
        np.savez_compressed(HERE / f"{name}.npz", **fn())
        print(name, (HERE / f"{name}.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
