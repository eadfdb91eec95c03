"""Multi-GPU runs are independent replicas: the only cross-rank work is the
barrier and the max-over-ranks timing of bench.py.  Checked here with two
gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(world)
    elapsed = 1.0 + rank  # rank 1 is the slowest
    value, t = bench.aggregate(elapsed, 5, world)
    q.put((rank, value, t, bench.dist_env()))
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_replicas_aggregate_over_slowest_rank():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=90) for _ in range(world)]
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank, value, t, env in out:
        assert t == 2.0
        assert value == pytest.approx(world * 5 / 2.0)
        assert env == (world, rank, rank)


def test_single_process_aggregate():
    import bench
    value, t = bench.aggregate(0.5, 4, 1)
    assert t == 0.5 and value == 8.0
