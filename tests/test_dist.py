"""The N > 1 bench path on CPU: world-size-2 gloo process groups (127.0.0.1)
running bench.Dist (barrier, max and sum over ranks: the timing and
whole-job throughput of the multi-GPU line), and the round-robin sharding of
the batched realisations (disjoint, complete, no data-path exchange)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path[:0] = [str(ROOT), str(ROOT / "gpe-matlab_gb300")]
    import bench
    from gpe_workloads import BATCH2D

    d = bench.Dist()
    d.barrier()
    s = d.reduce(float(rank + 1), "sum")
    m = d.reduce(float(10 * rank), "max")
    mine = BATCH2D.shard(rank, world)
    tot = d.reduce(float(len(mine)), "sum")
    d.close()
    out.put((rank, s, m, tot, mine))


def test_two_rank_gloo_reductions_and_sharding():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, s, m, tot, mine in res:
        assert s == 3.0 and m == 10.0 and tot == 64.0
    a, b = res[0][4], res[1][4]
    assert not set(a) & set(b) and sorted(a + b) == list(range(64))
