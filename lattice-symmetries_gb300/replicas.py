"""Host-side logic for running the hot path on several GPUs of one node, one process per GPU.

The path does not exchange data between GPUs: independent symmetry sectors (or independent
copies of one workload) are assigned to ranks, and only timings and scalar results are combined
(`torch.distributed` with NCCL on GPUs, gloo on CPU).  This is the GPU counterpart of the
reference's split of the work among locales (chapel/src/StatesEnumeration.chpl:392-458), with
whole sectors as the unit: every sector fits one GB300, so no state is hashed to another GPU and
no exchange of (beta, c) pairs is needed (the reference's DistributedMatrixVector.chpl:179-339).
"""

from __future__ import annotations

import heapq
from typing import Any, Dict, List, Sequence, Tuple


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


def world_and_rank() -> Tuple[int, int]:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist.get_world_size(), dist.get_rank()
    return 1, 0


def my_units(weights: Sequence[float]) -> List[int]:
    """This rank's share of the units (shard_by_weight over the process group; all units when no
    group is initialised)."""
    world, rank = world_and_rank()
    return shard_by_weight(weights, world)[rank]


def gather_results(local: Dict[int, Any]) -> Dict[int, Any]:
    """Merges every rank's {unit: result} into one dict (all ranks receive it); a unit reported
    twice is an error."""
    import torch.distributed as dist
    world, _ = world_and_rank()
    if world == 1:
        return dict(local)
    parts: List[Any] = [None] * world
    dist.all_gather_object(parts, dict(local))
    out: Dict[int, Any] = {}
    for part in parts:
        for k, v in part.items():
            if k in out:
                raise RuntimeError("unit {} reported by two ranks".format(k))
            out[k] = v
    return out
