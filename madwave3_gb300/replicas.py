"""Multi-GPU layer: partial waves are independent, so N GPUs split the waves of
a sweep (or run N replicas of one wave) with no data-path exchange.  Only the
host side talks across ranks: the timing reduction (max over ranks) and the
gather of per-wave results to rank 0.  torch.distributed carries these; any
backend works (nccl on GPUs, gloo on CPUs).
"""
import heapq


def partition(costs, world):
    """Longest-processing-time assignment of waves to ranks.

    costs[i] is the work of wave i (e.g. blocks x stored points); returns a list
    of wave-index lists, one per rank, each sorted ascending."""
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(x) for x in out]


def max_over_ranks(value):
    """Largest float over all ranks (the step time the job waits for)."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_results(local):
    """Merge {wave_key: result} dicts of all ranks on rank 0 (None elsewhere)."""
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return dict(local)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, local)
    if dist.get_rank() != 0:
        return None
    merged = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise ValueError("wave %r computed on two ranks" % (k,))
            merged[k] = v
    return merged
