"""Host logic of the N>1 replica path on CPU: world_size-2 gloo ranks."""
import os
import socket

import pytest

from vca_gb300.replicas import Group, partition


def test_partition_covers_every_point_once():
    for n in (1, 7, 16):
        for world in (1, 2, 3, 8):
            seen = sorted(i for r in range(world) for i in partition(n, r, world))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        partition(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    g = Group(dist)
    idx = partition(16, rank, world)
    vals = [100.0 + i for i in idx]
    g.barrier()
    tmax = g.max(1.0 + rank)
    allv = g.gather_values(idx, vals, 16)
    dist.destroy_process_group()
    q.put((rank, tmax, allv))


def test_gloo_two_ranks_max_and_gather():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tmax, allv in res:
        assert tmax == 2.0
        assert allv == [100.0 + i for i in range(16)]
