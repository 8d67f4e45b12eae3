"""Multi-GPU host logic: replicas with disjoint frame numbers, no collective on
the data path (pixels, samples and jobs are independent: weak scaling). Only
the timing/ray totals are reduced, after the timed region.

frame_number(step, rank, world) gives every rank its own State.frameCount
stream, so N ranks rendering K steps produce N*K distinct passes of one image
(together the same progressive render one GPU would make in N*K steps).
"""
from __future__ import annotations


def frame_number(step: int, rank: int, world: int) -> float:
    return float(1 + step * world + rank)


def assign_requests(costs, world: int):
    """Served mode over N replicas: the rank that serves each request, in arrival
    order, given each request's cost (pixels x spp, the work its frame passes
    cost). Each request goes to the replica with the least work assigned so far
    (ties: the lower rank). Every replica holds every scene resident (BVHs are
    read-only) and runs its own merged-queue server; a request's film comes back
    from the one replica that rendered it, so no film is ever reduced across
    ranks."""
    load = [0.0] * world
    out = []
    for c in costs:
        r = min(range(world), key=lambda k: (load[k], k))
        out.append(r)
        load[r] += float(c)
    return out


def reduce_max_sum(seconds: float, rays: int, device=None):
    """(max over ranks of seconds, sum over ranks of rays) through torch.distributed;
    identity when no process group is initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return seconds, rays
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    r = torch.tensor([float(rays)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(r, op=dist.ReduceOp.SUM)
    return float(t.item()), int(r.item())
