"""Multi-process host logic (replicas, sector sharding) with world_size 2 over gloo on CPU."""

import importlib
import os
import socket

import pytest

torch = pytest.importorskip("torch")
rep = importlib.import_module("lattice-symmetries_gb300.replicas")


def test_shard_by_weight_covers_and_balances():
    weights = [716728, 716200, 715000, 700, 50, 50, 50, 9000, 9000, 12]
    for world in (1, 2, 3, 4, 8):
        parts = rep.shard_by_weight(weights, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(weights)))
        loads = [sum(weights[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(weights)
    assert rep.shard_by_weight(weights, 2) == rep.shard_by_weight(list(weights), 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, queue):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rep.barrier()
        slowest = rep.max_over_ranks(10.0 * (rank + 1))
        total = rep.sum_over_ranks(rank + 1)
        mine = rep.shard_by_weight([5, 4, 3, 2, 1, 1], world)[rank]
        all_parts = [None] * world
        dist.all_gather_object(all_parts, mine)
        queue.put((rank, slowest, total, all_parts))
    finally:
        dist.destroy_process_group()


def test_two_ranks_over_gloo():
    mp = torch.multiprocessing.get_context("spawn")
    queue = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = [queue.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, total, parts in results:
        assert slowest == 20.0
        assert total == 3.0
        assert sorted(i for p in parts for i in p) == list(range(6))
        assert parts == rep.shard_by_weight([5, 4, 3, 2, 1, 1], 2)
