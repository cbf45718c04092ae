#!/usr/bin/env python3
"""Benchmark: FSSH spin-boson ensemble throughput on GB300 (traj-steps/s).

Workload (one "step" of this benchmark = one full ensemble run): Ohmic
spin-boson, 100 bath modes, 100 000 trajectories, dt = 0.05, t in [0, 20]
(400 nuclear steps) = 4.0e7 trajectory-steps, diabatic population
correlation saved every 0.1.  Synthetic seeded inputs with the reference
configuration's shapes (nqcd_gb300/workload.py).

  value      chosen (FP32) path, inputs resident in HBM, CUDA-event time of
             the engine's work on its stream
  e2e        same metric through the C ABI with host buffers: nqcd_set_initial
             (host->device + layout gather) + nqcd_run (+ observables back)
  plain_fp64 plain FP64 path (bit-identical to the FP64 oracle), same inputs
  cpu_baseline  the CPU oracle (FP64 restatement of the reference) on the
             host cores, on a bounded sample of the same workload

--impl reference times the CPU restatement of the reference integration on
the host cores (the reference itself is Julia and cannot run here).
Multi-GPU (torchrun): each rank runs an independent replica shard of
trajectories (global trajectory ids offset by rank); no collective on the
data path, only a barrier and a max over ranks of the timings.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "nqcdynamics.jl_gb300"))

WORKLOAD = "fssh_spinboson_ohmic100_traj100k_dt0.05_t20"
METRIC = "traj-steps/s on 1 GB300: chosen vs plain FP64 path at stated observable error"
UNIT = "traj-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ntraj", type=int, default=100_000)
    ap.add_argument("--nmodes", type=int, default=100)
    ap.add_argument("--t1", type=float, default=20.0)
    ap.add_argument("--dt", type=float, default=0.05)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (barrier + max over ranks only)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# engine helpers
# ---------------------------------------------------------------------------
def make_engine(L, prec, w, c, ntraj, nmodes, save_stride, traj_offset):
    cfg = L.nqcd_config()
    cfg.method, cfg.model, cfg.precision = L.METHOD_FSSH, L.MODEL_SPINBOSON, prec
    cfg.rescaling = 0
    cfg.ndofs, cfg.natoms, cfg.nstates = 1, nmodes, 2
    params = np.array([0.0, 1.0])
    masses = np.ones(nmodes)
    cfg.nparams, cfg.params, cfg.masses = 2, L.dptr(params), L.dptr(masses)
    cfg.nbath, cfg.bath_a, cfg.bath_b = nmodes, L.dptr(c), L.dptr(w)
    cfg.ntraj_max = ntraj
    cfg.init_kind, cfg.init_state = L.INIT_DIABATIC_PURE, 0
    cfg.save_stride = save_stride
    cfg.max_hops = 0
    cfg.gap_fp64 = 1e-3
    cfg.traj_offset = traj_offset
    return L.Engine(cfg, [params, masses, c, w])


def time_engine(eng, steps, warmup, t1, dt, seed, popcorr, dist):
    for _ in range(warmup):
        eng.run(0.0, t1, dt, seed, popcorr=popcorr)
    dist.barrier()
    dev, ker, traj_steps, launches = 0.0, [], 0, 0
    w0 = time.perf_counter()
    for _ in range(steps):
        _, st = eng.run(0.0, t1, dt, seed, popcorr=popcorr)
        dev += st.device_ms
        ker.append(st.kernel_ms)
        traj_steps += st.traj_steps
        launches += st.kernel_launches
    wall = time.perf_counter() - w0
    dist.barrier()
    return dict(device_ms=dev, kernel_ms=ker, traj_steps=traj_steps, launches=launches, wall_s=wall)


def cpu_baseline(args, w, c, r0, v0, nthreads):
    """Bounded sample of the same workload through the CPU oracle."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    def run(n):
        t = time.perf_counter()
        O.run_fssh(model=10, params=(0.0, 1.0), ndof=args.nmodes, mass=1.0, r0=r0[:n], v0=v0[:n], t0=0.0,
                   t1=args.t1, dt=args.dt, seed=20261203, init_kind=2, init_state=0, bath_c=c, bath_w2=w * w,
                   save_stride=int(round(0.1 / args.dt)), max_hops=0, nthreads=nthreads)
        return time.perf_counter() - t

    n = min(len(r0), max(nthreads * 4, 64))
    s = run(n)
    n2 = int(min(len(r0), max(n, n * args.cpu_seconds / max(s, 1e-3))))
    if n2 > n:
        s = run(n2)
        n = n2
    nsteps = int(round(args.t1 / args.dt))
    return {"value": n * nsteps / s, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{n} of {args.ntraj} trajectories x {nsteps} steps (full length), {s:.1f} s"}


def main():
    args = parse()
    dist = Dist()
    from nqcd_gb300 import build as B
    from nqcd_gb300 import workload as WL

    if args.impl == "reference":
        return reference_arm(args, dist, B, WL)

    B.build_all()
    from nqcd_gb300 import _lib as L

    nmodes, ntraj = args.nmodes, args.ntraj
    traj_offset = dist.rank * ntraj
    w, c, r0, v0 = WL.spin_boson_inputs(ntraj, nmodes, traj_offset=traj_offset)
    save_stride = int(round(0.1 / args.dt))
    nsteps = int(round(args.t1 / args.dt))
    nsave = nsteps // save_stride + 1
    seed = WL.SEED

    fp64_peak, fp32_peak = L.measure_fma_peaks()

    # plain FP64 path first: the reference for the observable error of the fast paths
    paths = {}
    for name, prec, nsteps_t in (("fp64", L.PREC_FP64, max(1, args.fp64_steps)),
                                 ("fp32", L.PREC_FP32, args.steps),
                                 ("fp32_kahan", L.PREC_FP32_KAHAN, args.steps)):
        eng = make_engine(L, prec, w, c, ntraj, nmodes, save_stride, traj_offset)
        eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0))
        pc = np.zeros(nsave * 4)
        with ClockSampler(dist.local) as clk:
            tm = time_engine(eng, nsteps_t, args.warmup if name != "fp64" else 1, args.t1, args.dt, seed, pc, dist)
        tm["clocks"] = clk.summary()
        tm["popcorr"] = pc.reshape(nsave, 4)
        tm["engine"] = eng
        tm["steps"] = nsteps_t
        tm["dev_s"] = dist.max(tm["device_ms"] / 1e3)
        tm["value"] = dist.sum(tm["traj_steps"]) / tm["dev_s"]
        paths[name] = tm
    ref = paths["fp64"]["popcorr"]
    for name, tm in paths.items():
        d = tm["popcorr"][:, 0] - tm["popcorr"][:, 1]
        dref = ref[:, 0] - ref[:, 1]
        tm["obs_err"] = float(np.max(np.abs(d - dref)))
    OBS_TOL = 0.01  # 1% of the population-difference range
    ok = [n for n in ("fp32_kahan", "fp32") if paths[n]["obs_err"] <= OBS_TOL]
    chosen = max(ok, key=lambda n: paths[n]["value"]) if ok else "fp64"
    ch = paths[chosen]
    clocks = ch["clocks"]
    eng32 = ch["engine"]
    pc32 = np.zeros(nsave * 4)

    # e2e through the C ABI with pinned host buffers, copies inside the timed region
    e2e = None
    if not args.no_e2e:
        r0c, v0c = np.ascontiguousarray(r0), np.ascontiguousarray(v0)
        lib = L.load()
        lib.nqcd_pin_host(r0c.ctypes.data, r0c.nbytes)
        lib.nqcd_pin_host(v0c.ctypes.data, v0c.nbytes)
        eng32.set_initial(r0c, v0c)
        eng32.run(0.0, args.t1, args.dt, seed, popcorr=pc32)
        dist.barrier()
        t0 = time.perf_counter()
        ts = 0
        d2h = 0
        for _ in range(args.steps):
            eng32.set_initial(r0c, v0c)
            _, st = eng32.run(0.0, args.t1, args.dt, seed, popcorr=pc32)
            ts += st.traj_steps
            d2h += st.d2h_bytes
        el = dist.max(time.perf_counter() - t0)
        dist.barrier()
        lib.nqcd_unpin_host(r0c.ctypes.data)
        lib.nqcd_unpin_host(v0c.ctypes.data)
        e2e = {"value": dist.sum(ts) / el, "unit": UNIT, "h2d_bytes_per_step": int(r0c.nbytes + v0c.nbytes),
               "d2h_bytes_per_step": int(d2h // args.steps)}
    for tm in paths.values():
        tm["engine"].close()

    value = ch["value"]
    plain = paths["fp64"]["value"]
    ker_ms = float(np.mean(ch["kernel_ms"]))
    flops_launch = WL.ref_flops_per_traj_step(nmodes) * ntraj * nsteps
    achieved = flops_launch / (ker_ms * 1e-3) / 1e12
    hbm_bytes = 2 * 2 * ntraj * nmodes * 8  # r, v read + written once per run by an on-chip kernel
    kname = {"fp64": "fssh2_spinboson_kernel<double>", "fp32": "fssh2_sb_fast_kernel<AccF64,25>",
             "fp32_kahan": "fssh2_sb_fast_kernel<AccKahan,25>"}[chosen]
    roofline = {"bound": "fp32-core" if chosen != "fp64" else "fp64-core", "achieved": achieved,
                "peak": fp32_peak if chosen != "fp64" else fp64_peak, "unit": "TFLOP/s",
                "traffic": None,
                "peak_source": "measured FMA throughput (project microbenchmark); MEASURED_PEAKS has no CUDA-core entry",
                "flops_per_traj_step": WL.ref_flops_per_traj_step(nmodes), "kernel": kname,
                "kernel_ms": ker_ms, "hbm_peak_gbs": 6751.1,
                "algorithmic_hbm_gbs": hbm_bytes / (ker_ms * 1e-3) / 1e9}
    roofline["frac"] = roofline["achieved"] / roofline["peak"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ch["dev_s"] * 1e3 / ch["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32_kahan": "fp32+kahan-acc", "fp32": "fp32+fp64acc", "fp64": "f64"}[chosen],
        "data": "synthetic", "chosen_path": chosen,
        "config": {"workload": WORKLOAD, "ntraj_per_gpu": ntraj, "modes": nmodes, "nsteps": nsteps,
                   "traj_steps_per_step": ntraj * nsteps, "parallelism": f"replicas{dist.world}",
                   "l2": "inputs larger than L2 (positions+velocities 160 MB)"},
        "paths": {n: {"value": tm["value"], "ms_per_step": tm["dev_s"] * 1e3 / tm["steps"],
                      "kernel_ms": float(np.mean(tm["kernel_ms"])), "observable_error": tm["obs_err"],
                      "speedup_vs_plain_fp64": tm["value"] / plain} for n, tm in paths.items()},
        "plain_fp64": {"value": plain, "unit": UNIT, "speedup_chosen_vs_plain": value / plain},
        "observable_error": {"quantity": "max_t |<P1-P2>(t)| chosen - plain FP64 (population-difference correlation)",
                             "value": ch["obs_err"], "tolerance": OBS_TOL, "ntraj": ntraj},
        "e2e": e2e,
        "roofline": roofline,
        "peaks_measured": {"fp64_tflops": fp64_peak, "fp32_tflops": fp32_peak},
        "clocks": clocks,
        "gpu_launches": ch["launches"],
    }
    if dist.rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args, w, c, r0, v0, os.cpu_count() or 1)
    if dist.rank == 0:
        print(json.dumps(line))


def reference_arm(args, dist, B, WL):
    if dist.rank != 0:
        return
    B.build_oracle()
    nmodes, ntraj = args.nmodes, args.ntraj
    w, c, r0, v0 = WL.spin_boson_inputs(ntraj, nmodes)
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    nthreads = os.cpu_count() or 1
    nsteps = int(round(args.t1 / args.dt))
    # bounded sample per step: enough trajectories for ~ (budget / steps) seconds
    budget = 120.0 / max(1, args.steps + args.warmup)
    probe_n = min(ntraj, nthreads * 8)
    t = time.perf_counter()
    O.run_fssh(model=10, params=(0.0, 1.0), ndof=nmodes, mass=1.0, r0=r0[:probe_n], v0=v0[:probe_n], t0=0.0,
               t1=args.t1, dt=args.dt, seed=WL.SEED, init_kind=2, bath_c=c, bath_w2=w * w,
               save_stride=int(round(0.1 / args.dt)), max_hops=0, nthreads=nthreads)
    per = (time.perf_counter() - t) / probe_n
    n = int(min(ntraj, max(probe_n, budget / max(per, 1e-9))))
    times = []
    for it in range(args.warmup + args.steps):
        t = time.perf_counter()
        O.run_fssh(model=10, params=(0.0, 1.0), ndof=nmodes, mass=1.0, r0=r0[:n], v0=v0[:n], t0=0.0, t1=args.t1,
                   dt=args.dt, seed=WL.SEED, init_kind=2, bath_c=c, bath_w2=w * w,
                   save_stride=int(round(0.1 / args.dt)), max_hops=0, nthreads=nthreads)
        if it >= args.warmup:
            times.append(time.perf_counter() - t)
    tot = sum(times)
    value = n * nsteps * len(times) / tot
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot * 1e3 / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "ntraj_per_gpu": ntraj, "modes": nmodes, "nsteps": nsteps},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{n} of {ntraj} trajectories x {nsteps} steps per step; the reference is Julia "
                                   f"(no Julia toolchain), so its FP64 integration is timed through the CPU "
                                   f"restatement"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
