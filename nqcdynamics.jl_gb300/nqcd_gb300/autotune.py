"""Project autotuner for the fast kernels' launch shapes (nqcd_set_mapping).

For a workload it times every candidate mapping on the GPU with the
engine's own kernel timing (CUDA events around the ensemble kernel,
nqcd_stats.kernel_ms; best of a few runs after a warm-up run), keeps the
fastest, and caches the sweep in JSON keyed by GPU (name and SM count) and
workload:

  spin-boson FSSH, Kahan-accumulated fast kernel: lanes per trajectory
      (4, 8) x threads per block (64, 128, 256);
  ring-polymer FSSH: lanes per trajectory of each bead count's kernel
      (4 beads: 1, 2, 4; 8: 2, 4, 8; 16: 4, 8, 16; 32: 4, 8, 16, 32), by
      coordinate descent on the mixed C3 ensemble of 200 000 trajectories (the four kernels run
      concurrently, so a shape is judged by the whole ensemble's time), and
      against it one persistent launch serving every bead count.

The committed cache (tuned/mappings.json) holds the sweeps measured on a
GB300; NQCD_TUNE_CACHE names another file.  `mapping_for` returns the cached
mapping or, for a GPU or workload not in the cache, runs the sweep first.

    python -m nqcd_gb300.autotune [spinboson|rpsh|all]
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

from . import configs as C
from . import workload as WL

CACHE = Path(os.environ.get("NQCD_TUNE_CACHE", Path(__file__).resolve().parent / "tuned" / "mappings.json"))

SB_LANES = (4, 8)
SB_BLOCKS = (64, 128, 256)
RP_LANES = {4: (1, 2, 4), 8: (2, 4, 8), 16: (4, 8, 16), 32: (4, 8, 16, 32)}


def gpu_key() -> str:
    import torch

    p = torch.cuda.get_device_properties(0)
    return f"{p.name}|{p.multi_processor_count}"


def load() -> dict:
    return json.loads(CACHE.read_text()) if CACHE.exists() else {}


def save(db: dict) -> None:
    CACHE.parent.mkdir(parents=True, exist_ok=True)
    CACHE.write_text(json.dumps(db, indent=1, sort_keys=True) + "\n")


def _best_kernel_ms(eng, run, repeats):
    run()  # warm-up
    return min(run()[1].kernel_ms for _ in range(repeats))


def tune_spinboson(L, ntraj=100_000, nmodes=100, t1=20.0, dt=0.05, repeats=3):
    """Sweep of the spin-boson fast kernel (Kahan accumulators) on the
    headline ensemble; returns (best mapping dict, sweep rows)."""
    w, c, r0, v0 = WL.spin_boson_inputs(ntraj, nmodes)
    eng = C.spinboson_fssh(L, w, c, ntraj, nmodes, L.PREC_FP32_KAHAN)
    rows = []
    try:
        eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0))
        for lanes in SB_LANES:
            if lanes == 8 and nmodes > 128:
                continue
            for block in SB_BLOCKS:
                eng.set_mapping(dict(sb_lanes=lanes, sb_block=block))
                ms = _best_kernel_ms(eng, lambda: eng.run(0.0, t1, dt, WL.SEED), repeats)
                rows.append(dict(sb_lanes=lanes, sb_block=block, kernel_ms=ms,
                                 traj_steps_per_s=ntraj * round(t1 / dt) / (ms / 1e3)))
    finally:
        eng.close()
    best = min(rows, key=lambda r: r["kernel_ms"])
    return dict(sb_lanes=best["sb_lanes"], sb_block=best["sb_block"]), rows


def tune_rpsh(L, ntraj=200_000, repeats=2):
    """Sweep of the ring-polymer fast kernels on the mixed ring-polymer
    benchmark ensemble (Tully 1-3 round robin, bead counts 4-32 mixed,
    termination at |x| > 10), where the four bead-count kernels run
    concurrently and share the SMs: coordinate descent from the defaults,
    one bead count at a time over its lane groups with the others fixed.
    The sweep runs at the ensemble's own size: on a quarter of it the tail
    of the 32-bead class dominates and favours wider lane groups, which
    lose throughput on the full ensemble.
    Returns (best rp_lanes dict, sweep rows)."""
    r0, v0, nb, models = C.rpsh_inputs(ntraj)
    eng = C.rpsh_tully(L, ntraj, L.PREC_FP32)
    best = {b: 4 for b in RP_LANES}
    rows = []
    try:
        eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0), nbeads=np.ascontiguousarray(nb))
        eng.set_trajectory_models(np.ascontiguousarray(models))
        timed = {}

        def time_of(mp):
            key = tuple(sorted(mp.items()))
            if key not in timed:
                eng.set_mapping(dict(rp_lanes=mp))
                timed[key] = _best_kernel_ms(eng, lambda: eng.run(0.0, 20000.0, 1.0, WL.SEED), repeats)
                rows.append(dict(rp_lanes={str(k): v for k, v in mp.items()}, kernel_ms=timed[key]))
            return timed[key]

        for beads, cands in RP_LANES.items():
            trial = {lanes: time_of({**best, beads: lanes}) for lanes in cands}
            best[beads] = min(trial, key=trial.get)
        # one persistent launch for every bead count (default lane groups) against the
        # concurrent per-bead-count kernels
        eng.set_mapping(dict(rp_one_launch=1))
        one_ms = _best_kernel_ms(eng, lambda: eng.run(0.0, 20000.0, 1.0, WL.SEED), repeats)
        rows.append(dict(rp_one_launch=1, kernel_ms=one_ms))
    finally:
        eng.close()
    if one_ms < time_of(best):
        return dict(rp_one_launch=1), rows
    return dict(rp_lanes=best), rows


TUNERS = {"spinboson": tune_spinboson, "rpsh": tune_rpsh}


def workload_key(workload: str, **kw) -> str:
    if workload == "spinboson":
        return f"spinboson_modes{kw.get('nmodes', 100)}_traj{kw.get('ntraj', 100_000)}"
    return f"rpsh_tully123_mixed_traj{kw.get('ntraj', 200_000)}"


def tune(L, workload: str, **kw) -> dict:
    """Run the sweep of `workload`, store it in the cache and return the entry."""
    t = time.perf_counter()
    best, rows = TUNERS[workload](L, **kw)
    entry = dict(mapping=best, sweep=rows, seconds=time.perf_counter() - t,
                 when=time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()))
    db = load()
    db.setdefault(gpu_key(), {})[workload_key(workload, **kw)] = entry
    save(db)
    return entry


def mapping_for(L, workload: str, allow_tune: bool = True, **kw):
    """(mapping dict, source) for this GPU and workload: the cached sweep's
    winner, or the winner of a sweep run now (and cached); the defaults when
    the cache has no entry and tuning is not allowed (several ranks)."""
    entry = load().get(gpu_key(), {}).get(workload_key(workload, **kw))
    if entry is not None:
        return _keys_to_int(entry["mapping"]), f"autotune cache {CACHE.name}"
    if not allow_tune:
        return {}, "defaults (no cached sweep for this GPU)"
    entry = tune(L, workload, **kw)
    return _keys_to_int(entry["mapping"]), "autotune sweep run now"


def _keys_to_int(m: dict) -> dict:
    out = dict(m)
    if "rp_lanes" in out:
        out["rp_lanes"] = {int(k): int(v) for k, v in out["rp_lanes"].items()}
    return out


def main(argv):
    from . import build as B

    B.build_all()
    from . import _lib as L

    which = argv[0] if argv else "all"
    for wk in (TUNERS if which == "all" else [which]):
        entry = tune(L, wk)
        print(wk, json.dumps(entry["mapping"]), f"{entry['seconds']:.1f} s")
        for row in entry["sweep"]:
            print("  ", row)


if __name__ == "__main__":
    main(sys.argv[1:])
