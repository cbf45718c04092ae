"""Multi-GPU decomposition (replicas only), tested on CPU with two gloo ranks.

Trajectories are independent and the random stream is keyed by the global
trajectory index, so a sharded ensemble (rank r takes trajectories
[r n, (r + 1) n) with traj_offset = r n) summed over ranks equals the
single-process ensemble exactly.  The ranks here run the CPU oracle on their
shards and combine their accumulators with one all_reduce, as bench.py's
replicas combine trajectory counts; no GPU is involved.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

NTRAJ = 64
T1 = (0.01, 1.6, 0.005, 1.0)


def _inputs():
    rng = np.random.default_rng(11)
    r0 = np.full((NTRAJ, 1), -10.0)
    v0 = rng.uniform(8.0, 30.0, (NTRAJ, 1)) / 2000.0
    return r0, v0


def _accumulators(res):
    """Sums that a replica contributes: state-resolved scattering counts, hop
    and frustrated-hop totals and the sum of final positions."""
    x = res["r"][:, 0]
    st = res["state"]
    counts = np.array([np.sum((x < 0) & (st == 0)), np.sum((x < 0) & (st == 1)),
                       np.sum((x > 0) & (st == 0)), np.sum((x > 0) & (st == 1))], dtype=np.float64)
    return np.concatenate([counts, [res["nhops"].sum(), res["nfrustrated"].sum(), x.sum()]])


def _run(offset, n, r0, v0):
    import oracle as O

    return O.run_fssh(model=1, params=T1, ndof=1, mass=2000.0, r0=r0[offset:offset + n], v0=v0[offset:offset + n],
                      t0=0.0, t1=3000.0, dt=1.0, seed=20261203, traj_offset=offset, max_hops=16, nthreads=1)


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r0, v0 = _inputs()
        n = NTRAJ // world
        res = _run(rank * n, n, r0, v0)
        acc = torch.tensor(_accumulators(res), dtype=torch.float64)
        dist.all_reduce(acc, op=dist.ReduceOp.SUM)
        tmax = torch.tensor([float(rank + 1)], dtype=torch.float64)
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)  # the timing reduction of bench.py
        if rank == 0:
            q.put((acc.numpy().tolist(), float(tmax.item())))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_sum_to_the_single_ensemble():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    acc, tmax = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    r0, v0 = _inputs()
    single = _accumulators(_run(0, NTRAJ, r0, v0))
    np.testing.assert_array_equal(np.array(acc[:6]), single[:6])
    assert acc[6] == pytest.approx(single[6], rel=1e-12)
    assert tmax == 2.0
