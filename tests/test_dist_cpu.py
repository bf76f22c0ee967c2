"""The multi-GPU host path of bench.py on CPU: two gloo ranks.

bench.py --gpus N runs N independent replicas; its process group only
brackets the timed region with barriers and combines the per-rank results
(max of the times, sum of the work).  These ranks run that logic on the host
(gloo, 127.0.0.1), and check that served requests are drawn from different
seeds on different ranks (independent replicas, no shared work).
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(backend="gloo")
    d.barrier()
    mx = d.reduce(10.0 * (rank + 1), "max")
    sm = d.reduce(rank + 1, "sum")
    import numpy as np
    from ddevol_gb300 import hamiltonians as H
    seed = bench.SERVE["seed"] + 7919 * d.rank  # as run_serve seeds each replica
    rng = np.random.default_rng(seed)
    sizes = [H.serving_request(rng)[0] for _ in range(8)]
    d.barrier()
    d.close()
    out.put((rank, mx, sm, seed, sizes))


def test_two_gloo_ranks_reduce_and_barrier():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in results] == [20.0, 20.0]  # max over ranks
    assert [r[2] for r in results] == [3.0, 3.0]    # sum over ranks
    assert results[0][4] != results[1][4]           # replicas draw different requests


def test_single_rank_is_a_no_op():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    d = bench.Dist()
    assert d.world == 1 and d.reduce(4.5, "max") == 4.5 and d.reduce(2, "sum") == 2
    d.barrier()
    d.close()
