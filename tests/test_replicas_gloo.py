"""Multi-GPU row: replicas only (patches of a level never exchange data inside a
substep), so bench.py's N > 1 path is N independent replicas whose timed region
is the slowest rank's.  This checks that aggregation with world_size 2 over the
gloo backend on the CPU: the max over ranks is taken and the whole-job value
counts every rank's cell-updates."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [120.0, 150.0][rank]
    total_ms, value = bench.replica_throughput(local_ms, cells_per_step=1000, steps=10, world=world, device="cpu")
    out.put((rank, total_ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, total_ms, value in res:
        assert total_ms == 150.0
        assert value == pytest.approx(2 * 1000 * 10 / 0.150)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.replica_throughput(200.0, 500, 4, 1, "cpu") == (200.0, 500 * 4 / 0.2)
