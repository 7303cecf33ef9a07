"""Multi-process path of bench.py on CPU: two gloo ranks (world size 2) reduce their replica
timings as the GPU bench does (max time over ranks, all ranks' paths), and a rank that raises is
seen by the launcher."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t_local = [0.5, 0.8][rank]
    paths = [1e6, 3e6][rank]
    t_max, rate = bench.replica_rate(t_local, paths, dist)
    q.put((rank, t_max, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, t_max, rate in got:
        assert t_max == pytest.approx(0.8)
        assert rate == pytest.approx(4e6 / 0.8 / 1e6)


def _failing_rank(rank: int, world: int, port: int) -> None:
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    if rank == 1:
        raise RuntimeError("rank 1 fails before joining")
    from datetime import timedelta
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=5))
    dist.destroy_process_group()


def test_a_failing_rank_is_reported():
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_failing_rank, args=(r, 2, port)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert procs[1].exitcode != 0          # the failure itself
    assert procs[0].exitcode != 0          # rank 0's rendezvous times out instead of hanging
