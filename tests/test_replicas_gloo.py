"""The bench's multi-GPU logic, world size 2 on gloo (CPU).

The path does not shard beyond independent replicas: each rank decodes its
own copy of the workload, the only collective is the MAX of the timed
regions, and the whole-job value is all ranks' fields over the slowest
rank's time. This runs the bench's own helpers in two gloo ranks.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_seconds = [0.5, 2.0][rank]            # rank 1 is the slow replica
    value, slowest = bench.replica_throughput(500, 5, local_seconds, dist, device="cpu")
    q.put((rank, value, slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_value_uses_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, value, slowest in res:
        assert slowest == pytest.approx(2.0)
        assert value == pytest.approx(500 * 5 * 2 / 2.0)


def test_single_process_needs_no_collective():
    import bench
    value, slowest = bench.replica_throughput(500, 5, 0.25, None)
    assert (value, slowest) == (pytest.approx(10000.0), 0.25)
