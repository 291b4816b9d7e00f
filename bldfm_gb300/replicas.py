"""Multi-GPU use: independent replicas over the case list.

Footprints are independent (the reference farms them to processes,
src/bldfm/interface.py:291-324), so N GPUs each solve a contiguous slice of
the cases with no collective on the data path; the results are gathered on the
host afterwards.  Works with any torch.distributed backend (NCCL between GPU
ranks, gloo on CPU).
"""

import torch.distributed as dist


def shard(n_cases, rank, world):
    """Contiguous slice [start, stop) of the cases owned by `rank`; slices are
    balanced to within one case and cover 0..n_cases-1 exactly once."""
    base, extra = divmod(n_cases, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop


def solve_sharded(cases, solve_fn, group=None):
    """Solve this rank's slice of `cases` with `solve_fn(list) -> list` and
    gather every rank's results on every rank, in case order (host objects;
    no device collective)."""
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    start, stop = shard(len(cases), rank, world)
    mine = solve_fn(cases[start:stop]) if stop > start else []
    if world == 1:
        return list(mine)
    parts = [None] * world
    dist.all_gather_object(parts, (start, list(mine)), group=group)
    out = []
    for s, res in sorted(parts, key=lambda x: x[0]):
        out.extend(res)
    return out


def max_time_ms(ms, device=None, group=None):
    """The slowest rank's time: the whole job's time for throughput."""
    if not dist.is_initialized() or dist.get_world_size(group) == 1:
        return ms
    import torch

    t = torch.tensor([float(ms)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
