"""Host-side logic for running the hot path on several GPUs of one node, one process per GPU.

The path does not exchange data between GPUs: independent symmetry sectors (or independent
copies of one workload) are assigned to ranks, and only timings and scalar results are combined
(`torch.distributed` with NCCL on GPUs, gloo on CPU).  The reference's distributed design (hashed
states and an all-to-all exchange per chunk, DistributedMatrixVector.chpl:179-339) is not used:
every sector fits one GB300.
"""

from __future__ import annotations

import heapq
from typing import List, Sequence


def shard_by_weight(weights: Sequence[float], world: int) -> List[List[int]]:
    """Assigns units (e.g. sectors with their sizes) to `world` ranks, largest first to the least
    loaded rank (LPT); every rank's list is ascending.  Deterministic for equal inputs."""
    if world < 1:
        raise ValueError("world must be positive")
    heap = [(0.0, r) for r in range(world)]
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i)):
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + float(weights[i]), r))
    return [sorted(p) for p in parts]


def _device():
    import torch
    import torch.distributed as dist
    return torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")


def max_over_ranks(value: float) -> float:
    """The maximum of `value` over all ranks (the time of the slowest replica)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()
