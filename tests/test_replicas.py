"""The N-GPU bench runs N independent replicas of the one-GPU workload (the path has no exchange step).

Its host logic is covered here on the CPU with gloo ranks, world size 2:
  * the job's step time is the maximum over ranks, taken after a barrier;
  * the reference arm runs on rank 0 only, and the other ranks return without work.
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


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r timed a mean of r + 1 and a worst step of 10 - r
        got = bench.max_over_ranks([rank + 1.0, 10.0 - rank])
        skipped = bench.run_reference(None) is None if rank != 0 else True
        with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
            f.write("%r %r %r\n" % (got[0], got[1], skipped))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_on_one_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]


def test_replica_timing_takes_the_slowest_rank(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        mean, worst, skipped = open(tmp_path / ("rank%d.txt" % r)).read().split()
        assert float(mean) == 2.0 and float(worst) == 10.0 and skipped == "True"
