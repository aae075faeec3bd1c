"""Multi-GPU sharding of the hot path (one process per GPU).

Pixels, views and frames are independent, so ranks split them with no
collective on the data path:
  * rendering: each rank takes a band of rows (or its own frame);
  * the differentiable marcher: each rank takes a subset of views, balanced
    by pixel count, and the per-view gradients are summed once per step
    (`allreduce_gradients`) -- the path's only exchange step.
"""
from __future__ import annotations

import heapq


def partition_views(pixel_counts: list[int], world_size: int) -> list[list[int]]:
    """Longest-processing-time assignment of views to ranks by pixel count;
    returns, per rank, its view indices in ascending order."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    heap = [(0, r) for r in range(world_size)]
    out: list[list[int]] = [[] for _ in range(world_size)]
    for i in sorted(range(len(pixel_counts)), key=lambda k: (-pixel_counts[k], k)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + pixel_counts[i], r))
    return [sorted(v) for v in out]


def row_band(height: int, world_size: int, rank: int) -> tuple[int, int]:
    """Rows [begin, end) of a frame rendered by `rank` (contiguous bands,
    sizes differing by at most one row)."""
    base, extra = divmod(height, world_size)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def allreduce_gradients(grads, group=None):
    """Sums gradient tensors across ranks in place (one all-reduce per
    tensor; works with gloo on CPU tensors and NCCL on CUDA tensors)."""
    import torch.distributed as dist

    for g in grads:
        dist.all_reduce(g, op=dist.ReduceOp.SUM, group=group)
    return grads
