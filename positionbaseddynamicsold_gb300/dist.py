"""Multi-GPU measurement helpers: one process per GPU.

A single cloth does not shard: its colored Gauss-Seidel is a chain of color
phases over shared points. N GPUs therefore run N independent replicas.
A batch of independent cloths does shard, by instance, with no exchange on
the data path: each rank simulates its share of the instances, and the
shares are balanced by point count. The only collective is the
max-over-ranks reduction of the measured time.
"""
from __future__ import annotations


def shard_instances(sizes, world: int, rank: int):
    """Indices of the instances `rank` simulates, ascending.

    Greedy and deterministic: instances in order of decreasing size (ties by
    index), each onto the least-loaded rank (ties by rank).
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world %d" % (rank, world))
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    load = [0] * world
    owner = [0] * len(sizes)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += sizes[i]
    return [i for i in range(len(sizes)) if owner[i] == rank]


def max_over_ranks(x: float) -> float:
    """The largest x over the ranks of the default process group (x itself
    without one). Ranks are synchronised after the reduction."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())
