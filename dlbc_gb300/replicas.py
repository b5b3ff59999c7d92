"""Multi-GPU use of the timestep: replicas, no exchange.

One lattice runs on one GPU (the domain is not decomposed, so the step has
no halo exchange to distribute).  Several GPUs run independent work:

* the same lattice on every rank (weak-scaling replicas of one workload);
* a batch of independent lattices split over the ranks by whole lattices
  (:func:`shard`), each rank stepping its share in its own batch.

The only collectives are on the host side, after the timed work: the
maximum time over ranks (:func:`max_over_ranks`) and the gathering of
per-rank records on rank 0 (:func:`gather_to_root`).  They work with any
torch.distributed backend (gloo on CPU, nccl on GPUs).
"""
from __future__ import annotations

import heapq
from typing import Any, List, Optional, Sequence


def shard(sizes: Sequence[int], world: int) -> List[List[int]]:
    """Assign items (by index) to `world` ranks so that the ranks' total
    sizes are balanced: largest item first to the least-loaded rank (LPT),
    ties to the lowest rank.  Every item goes to exactly one rank; each
    rank's list is in ascending index order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    heap = [(0, r) for r in range(world)]
    out: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(x) for x in out]


def max_over_ranks(value: float, dist: Optional[Any] = None, device: Optional[str] = None) -> float:
    """The maximum of `value` over all ranks (the value itself without a
    process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_root(obj: Any, dist: Optional[Any] = None) -> Optional[List[Any]]:
    """Every rank's `obj` as a list on rank 0 (None on the others); [obj]
    without a process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out
