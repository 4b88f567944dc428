"""The N-GPU benchmark path on CPU: two gloo ranks (world size 2) run the
host logic bench.py uses under torchrun — per-rank ensembles (seed + rank,
no data-path collective), barrier, max of the timed region over ranks and
sum of the work."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(
        os.path.abspath(__file__))))
    import bench
    from mbsolve_gb300 import setups
    d = bench.Dist(world)
    try:
        runs, params = setups.ensemble_2lvl(num_runs=8, seed=0 + d.rank)
        cells = int(params["num_gridpoints"].sum())
        d.barrier()
        t = 1.0 + d.rank          # this rank's timed region
        t_max = d.max(t)
        total = d.sum(cells)
        q.put((d.rank, cells, t_max, total,
               [float(x) for x in params["detuning"][:3]]))
    finally:
        d.close()


def test_two_gloo_ranks_shard_runs_and_reduce_timing():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q))
             for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=10) for _ in range(2))
    (r0, c0, t0, s0, d0), (r1, c1, t1, s1, d1) = res
    assert (r0, r1) == (0, 1)
    assert t0 == t1 == 2.0            # max over ranks
    assert s0 == s1 == c0 + c1        # whole-job work
    assert d0 != d1                   # each rank owns different runs
