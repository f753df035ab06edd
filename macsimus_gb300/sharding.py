"""Sharding of independent boxes over ranks (one GPU per rank).

Boxes are independent, so there is no data-path collective: each rank runs
its share of the boxes as one Batch and the per-box scalar results are
gathered on rank 0 over the host process group.  The share is balanced by an
estimated cost per box (r-space pairs plus k-space products)."""
import heapq


def box_cost(ns, nk, cutoff=None, L=None):
    """relative cost of one MD step of a box: k-space (ns x nk products) plus
    r-space (ns x sites within the cutoff, ~ the density times the sphere)"""
    pairs = ns * 200.0
    if cutoff is not None and L is not None:
        pairs = ns * ns * (4.18879 * cutoff ** 3) / (L ** 3)
    return ns * nk + 4.0 * pairs


def partition(costs, nranks):
    """longest-processing-time-first assignment: box indices per rank,
    each list ascending; deterministic for equal costs"""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(nranks)]
    heapq.heapify(heap)
    parts = [[] for _ in range(nranks)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(p) for p in parts]


def gather_results(local, rank, world):
    """{box index: result} of every rank merged on rank 0 (None elsewhere),
    over the default torch.distributed group (any backend)"""
    if world == 1:
        return dict(local)
    import torch.distributed as dist
    out = [None] * world if rank == 0 else None
    dist.gather_object(dict(local), out, dst=0)
    if rank != 0:
        return None
    merged = {}
    for d in out:
        for k, v in d.items():
            if k in merged:
                raise ValueError("box %d computed by two ranks" % k)
            merged[k] = v
    return merged
