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


def _sector_worker(rank, world, port, queue):
    """A rank of the sector split: its share of 56 sectors (LPT on their sizes), a host stand-in
    for the GPU step (a per-sector number that depends only on the sector), max-over-ranks time
    and the merged results."""
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = [716000 + 37 * ((s * 7919) % 101) for s in range(56)]
        mine = rep.my_units(sizes)
        local = {s: -0.5 * s + 1e-3 * sizes[s] for s in mine}  # stand-in for a sector's E0
        merged = rep.gather_results(local)
        slowest = rep.max_over_ranks(float(sum(sizes[s] for s in mine)))
        queue.put((rank, mine, merged, slowest))
    finally:
        dist.destroy_process_group()


def test_sector_split_over_two_ranks():
    mp = torch.multiprocessing.get_context("spawn")
    queue = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_sector_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sizes = [716000 + 37 * ((s * 7919) % 101) for s in range(56)]
    serial = {s: -0.5 * s + 1e-3 * sizes[s] for s in range(56)}
    (_, mine0, merged0, slow0), (_, mine1, merged1, slow1) = results
    assert sorted(mine0 + mine1) == list(range(56)) and not set(mine0) & set(mine1)
    assert merged0 == merged1 == serial
    assert slow0 == slow1 == max(sum(sizes[s] for s in mine0), sum(sizes[s] for s in mine1))
    # without a process group a single process takes every unit
    assert rep.my_units(sizes) == list(range(56))
    assert rep.gather_results({1: 2.0}) == {1: 2.0}
