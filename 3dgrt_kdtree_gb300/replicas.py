"""Multi-GPU form: scene replicas.

Any ray may touch any Gaussian, so the scene does not shard: every rank (one
process per GPU) holds the whole scene and renders its own views, and no
collective touches the render data.  The only cross-rank step is timing: a
step takes as long as the slowest rank, so per-step times are reduced with a
max before the job throughput is formed.
"""
from __future__ import annotations


def partition(n_items: int, rank: int, world: int) -> range:
    """Contiguous share of items [0, n_items) for `rank` of `world`: sizes
    differ by at most one, lower ranks take the extra items."""
    if world < 1 or not 0 <= rank < world or n_items < 0:
        raise ValueError("need 0 <= rank < world and n_items >= 0")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value: float, device=None) -> float:
    """Max of `value` over all ranks of the default process group (the value
    itself without one, or with one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, max_ms: float) -> float:
    """Whole-job units per second when each of `world` ranks processes
    `units_per_rank` units and the slowest takes `max_ms` milliseconds."""
    if max_ms <= 0:
        raise ValueError("max_ms must be positive")
    return units_per_rank * world / (max_ms * 1e-3)
