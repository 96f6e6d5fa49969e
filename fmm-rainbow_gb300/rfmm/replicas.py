"""Multi-GPU host logic: one process per GPU, no data-path collective.

A single scene has one global dependency (its octree), so the plain solve
does not shard; N GPUs run N independent replicas.  Batches of independent
scenes shard by scene: each rank owns a subset, balanced by body count.  The
only collectives are the bench's barrier and the reduction of its timing.
"""
from __future__ import annotations


def shard_scenes(sizes, world):
    """Longest-processing-time partition of scene indices over `world` ranks.

    Returns a list (per rank) of scene indices, each list sorted; every scene
    appears exactly once and the per-rank body totals differ by at most the
    largest scene.
    """
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    load = [0] * world
    owned = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owned[r].append(i)
        load[r] += sizes[i]
    return [sorted(o) for o in owned]


def reduce_throughput(local_work: float, local_seconds: float):
    """Whole-job throughput over the process group: total work / slowest rank."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return local_work / local_seconds, local_work, local_seconds
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    w = torch.tensor([float(local_work)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(w.item()) / float(t.item()), float(w.item()), float(t.item())
