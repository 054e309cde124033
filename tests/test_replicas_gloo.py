"""The multi-GPU path is "replicas only": each rank runs an independent copy
of the workload and bench.py reports the summed throughput, timed by the
slowest rank.  This checks the cross-rank aggregation with two gloo ranks on
the CPU (no GPU)."""
import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    el = bench.max_over_ranks(100.0 + 50.0 * rank, world)  # rank 1 is the slow replica
    q.put((rank, el, bench.replicas_value(20, world, el)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, el, value in out:
        assert el == pytest.approx(150.0)           # max over ranks
        assert value == pytest.approx(2 * 20 / 0.150)  # whole-job steps/s
