"""Multi-GPU sharding of the render path: one process per GPU, no collective on the data path.

* Path tracing shards by sample range: rank r renders launches [first, first + count) of the
  image (``sample_range``), seeding its renderer with ``Renderer.set_sample_index(first * spp)``;
  the only exchange is one sum of the FP64 accumulators at the end (``reduce_image``; NCCL on
  GPUs, gloo on CPU), after which every rank holds the single-GPU image up to FP64 summation
  order.
* Batched rendering shards by job (``assign_jobs``: longest-processing-time-first on each job's
  cost, pixels x spp x bounces), with no exchange at all.
* The traversal benchmark shards by ray batch (weak scaling).
ReSTIR DI couples neighbouring pixels within a frame, so it runs as replicas (one frame per rank).
"""
from __future__ import annotations

import heapq


def sample_range(rank: int, world: int, n_launches: int):
    """(first launch, number of launches) of rank's contiguous share; shares differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in 0..world-1")
    base, extra = divmod(n_launches, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def assign_jobs(costs, world: int):
    """Job indices per rank, greedily balancing the summed cost (largest jobs first)."""
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for j in sorted(range(len(costs)), key=lambda k: -costs[k]):
        load, r = heapq.heappop(heap)
        out[r].append(j)
        heapq.heappush(heap, (load + float(costs[j]), r))
    return [sorted(js) for js in out]


def reduce_image(image_sums, group=None):
    """Sums the ranks' FP64 accumulator arrays in place (torch.distributed all-reduce)."""
    import numpy as np
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(image_sums, np.float64))
    if dist.get_backend(group) == "nccl":
        d = t.cuda()
        dist.all_reduce(d, group=group)
        t = d.cpu()
    else:
        dist.all_reduce(t, group=group)
    return t.numpy()
