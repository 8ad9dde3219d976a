"""The multi-GPU bench runs independent replicas (one batch per rank, no
data-path collective): its timing takes the barrier and the maximum over
ranks.  Those two steps, run here as two gloo ranks on the CPU."""
import os
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, _ = bench.dist_setup()
        bench.barrier(ws)
        slowest = bench.reduce_max(1.5 + rank, ws)  # each rank's elapsed time
        q.put((got_rank, got_ws, slowest))
    finally:
        dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29000 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in procs)
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == pytest.approx(2.5) for r in res)
