"""Path sharding across ranks (weak or strong scaling) and the one exchange
step: an FP64 all-reduce of the per-rank payoff sums.

Paths are independent, so rank r of W simulates the global path range
[offset, offset + count) by passing ``path_offset = offset`` to the kernels:
Philox counters are global path indices, so the union of the shards is the
unsharded run.
"""

from __future__ import annotations

import torch


def shard_range(num_paths: int, rank: int, world: int) -> tuple[int, int]:
    """(offset, count) of rank's share of `num_paths` (strong scaling);
    the first num_paths % world ranks take one extra path."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank/world {rank}/{world}")
    base, extra = divmod(int(num_paths), int(world))
    count = base + (1 if rank < extra else 0)
    offset = rank * base + min(rank, extra)
    return offset, count


def weak_shard(paths_per_rank: int, rank: int) -> tuple[int, int]:
    """(offset, count) when every rank simulates `paths_per_rank` paths."""
    return rank * int(paths_per_rank), int(paths_per_rank)


def allreduce_sums(sums: torch.Tensor, group=None) -> torch.Tensor:
    """Sums FP64 accumulators across ranks in place (no-op without a process group)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(sums, op=dist.ReduceOp.SUM, group=group)
    return sums


__all__ = ["shard_range", "weak_shard", "allreduce_sums"]
