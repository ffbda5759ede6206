"""Multi-GPU is replicas only: every rank solves its own instances and the job
reports the maximum timed span over ranks and the solves of all ranks. The
host side of that path runs here as world_size-2 gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [250.0, 400.0][rank]           # rank 1 is the slower replica
    m = bench.max_over_ranks(ms, dist, "cpu")
    value = bench.replica_throughput(world, 16, 10, m)
    q.put((rank, m, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_max_over_ranks_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, value in got:
        assert m == 400.0
        assert value == pytest.approx(2 * 16 * 10 / 0.4)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(123.0, None) == 123.0
    assert bench.replica_throughput(1, 16, 10, 1000.0) == pytest.approx(160.0)
