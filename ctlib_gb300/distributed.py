"""Multi-GPU use: slices are independent, so a batch is split across ranks
(one process per GPU) with no exchange on the data path. The only collectives
are host-level bookkeeping: gathering results when a caller wants them on one
rank and reducing timings (max over ranks) in the benchmark.
"""

from __future__ import annotations

import torch


def shard_range(n: int, rank: int, world: int) -> tuple:
    """Contiguous [start, stop) of n slices owned by `rank` (sizes differ by at most 1)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard(x: torch.Tensor, rank: int, world: int) -> torch.Tensor:
    a, b = shard_range(x.shape[0], rank, world)
    return x[a:b]


def gather_shards(local: torch.Tensor, n: int, group=None) -> torch.Tensor:
    """All-gather the per-rank shards of an n-slice batch back into one tensor
    (ranks may hold different shard sizes)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    sizes = [shard_range(n, r, world) for r in range(world)]
    maxn = max(b - a for a, b in sizes)
    pad = torch.zeros((maxn,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[: local.shape[0]] = local
    bufs = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    return torch.cat([bufs[r][: sizes[r][1] - sizes[r][0]] for r in range(world)], dim=0)


def max_over_ranks(value: float, device=None, group=None) -> float:
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
