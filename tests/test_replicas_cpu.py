"""The multi-GPU path of bench.py on the CPU: a single SCD run does not shard, so
N GPUs run N independent replicas with no collective on the data path; the only
collective is the max of the step times over the ranks (the slowest replica sets
the job's time), and the job's rate is all the replicas' edges over that time.
Two gloo ranks on this machine stand in for two GPUs."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(dist, [10.0 + rank, 20.0 - 5 * rank], "cpu")
    out.put((rank, ms, bench.job_throughput(world, 1000, ms[0])))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for rank, ms, rate in got:
        assert ms == [11.0, 20.0]                 # the slowest rank's time, per value
        assert rate == pytest.approx(2 * 1000 / 0.011)


def test_one_process_keeps_its_values():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, [3.5, 4.0], "cpu") == [3.5, 4.0]
    assert bench.job_throughput(1, 500, 2.0) == pytest.approx(250000.0)
