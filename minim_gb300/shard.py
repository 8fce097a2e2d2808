"""Instance sharding across ranks (one process per GPU).

Independent minimisations need no exchange: instances are partitioned over
ranks by estimated cost (longest-processing-time greedy), each rank runs its
share with the batch kernels, and only the results are gathered on the host.
"""
import heapq


def instance_cost(kind, ndof, ndim=3):
    """Relative cost of one evaluation: pairs for Lennard-Jones, DOFs else."""
    if kind == 0:
        n = ndof // ndim
        return float(n) * n
    return float(ndof)


def partition(costs, world):
    """Assign item indices to `world` ranks, largest first onto the least
    loaded rank.  Deterministic: ties go to the lower rank / lower index."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(s) for s in out]


def gather(local, index, world, group=None):
    """Gather per-rank {index: result} onto every rank (torch.distributed
    object collective, host side only) and return them in global order."""
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, dict(zip(index, local)), group=group)
    merged = {}
    for p in parts:
        merged.update(p)
    return [merged[i] for i in sorted(merged)]
