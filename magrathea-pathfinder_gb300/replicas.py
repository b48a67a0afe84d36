"""Replica (data-parallel) layout of the propagation path over N GPUs.

Rays and cones are independent (one MPI rank per cone in the reference,
README "cone decomposition"; rays.cpp / hmaps.cpp give each rank its own
cones), so the path shards with no exchange on the data path: every rank
builds its own octree replica and traces its own share of the ray batches.
The only collectives are the timing barrier and the reductions of the
counters (max of the elapsed time, sum of the work), done here.
"""
from __future__ import annotations


def batch_ids(step: int, rank: int, world: int, n_batches: int) -> int:
    """Ray batch traced by `rank` at bench step `step`: ranks take interleaved
    batches, so N ranks cover N different batches per step."""
    return (step * world + rank) % n_batches


def shard(n_items: int, rank: int, world: int) -> slice:
    """Contiguous share of n_items for rank (sizes differ by at most one)."""
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def reduce_counters(dist, elapsed_ms: float, work: float, device=None):
    """(max elapsed over ranks, total work over ranks); identity without a process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(elapsed_ms), float(work)
    import torch
    t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
    w = torch.tensor([float(work)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())
