"""Multi-GPU is replicas only: every rank runs an independent world and the job's figure is
agent-hours summed over ranks over the slowest rank's time.  This runs bench.py's own
aggregation and seeding with two gloo ranks on the CPU (no GPU, no engine)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, root: str, out):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, root)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, agent_hours = 100.0 + 25.0 * rank, 1e9 * (rank + 1)
    ms_max, total = bench.aggregate_replicas(ms, agent_hours, "cpu")
    seeds = [None] * world
    dist.all_gather_object(seeds, bench.replica_seed(7, rank))
    if rank == 0:
        out.put((ms_max, total, seeds))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_replica_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, root, q)) for r in range(2)]
    for p in procs:
        p.start()
    ms_max, agent_hours, seeds = q.get(timeout=100)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ms_max == 125.0
    assert agent_hours == 3e9
    assert len(set(seeds)) == 2  # every rank simulates a different world
    value = agent_hours / (ms_max / 1000.0)  # the job's agent-hours/s
    assert value == pytest.approx(2.4e10)
