"""Splitting halo parts over ranks (one process per GPU).

Halo parts are independent: every triangle is counted in the part that owns
its lowest-ranked vertex, so ranks exchange nothing but one u64 sum at the
end.  Parts are assigned largest-first to the least-loaded rank (LPT), with a
part's work estimated by its oriented edge count unless given.
"""
from __future__ import annotations

from typing import Callable, Sequence


def assign_parts(work: Sequence[int], world: int) -> list[list[int]]:
    """Part indices for each rank, balancing the summed work (LPT)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for p in sorted(range(len(work)), key=lambda i: (-work[i], i)):
        r = min(range(world), key=lambda j: (load[j], j))
        out[r].append(p)
        load[r] += int(work[p])
    for lst in out:
        lst.sort()
    return out


def count_sharded(parts: Sequence, rank: int, world: int, count_fn: Callable[[object], int],
                  work: Sequence[int] | None = None, all_reduce_sum: Callable[[int], int] | None = None) -> int:
    """Counts this rank's share of `parts` with count_fn and returns the total
    over all ranks (all_reduce_sum combines the per-rank u64 partial sums; the
    default torch.distributed SUM works with gloo and nccl)."""
    w = list(work) if work is not None else [getattr(p, "nnz", 1) for p in parts]
    mine = assign_parts(w, world)[rank]
    local = sum(int(count_fn(parts[i])) for i in mine)
    if world == 1:
        return local
    if all_reduce_sum is None:
        import torch
        import torch.distributed as dist
        t = torch.tensor([local], dtype=torch.int64)
        if dist.get_backend() == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return int(t.item())
    return int(all_reduce_sum(local))
