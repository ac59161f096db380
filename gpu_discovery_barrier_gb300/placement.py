"""Graph -> GPU placement for the batched and serving forms on several GPUs.

A single traversal does not shard (every superstep needs the whole frontier
behind one grid barrier), but the batched and serving forms hold many
independent graphs: each graph goes to one GPU, whole, and the GPUs never
exchange data while they run -- only the results are gathered at the end.

Placement balances the arcs each GPU holds: members in decreasing order of
arcs, each to the GPU with the fewest arcs so far (longest-processing-time
first; ties go to the lower member index and the lower rank), so every
rank computes the same placement from the same sizes without talking to
the others.
"""
from __future__ import annotations

import heapq


def place(arcs, world: int) -> list[list[int]]:
    """Member indices per rank (each list ascending) for members of the
    given arc counts over `world` ranks."""
    if world < 1:
        raise ValueError("world must be at least 1")
    order = sorted(range(len(arcs)), key=lambda i: (-int(arcs[i]), i))
    heap = [(0, r) for r in range(world)]
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(arcs[i]), r))
    return [sorted(x) for x in out]


def owner_of(placement: list[list[int]]) -> dict[int, int]:
    """Member index -> rank."""
    return {i: r for r, members in enumerate(placement) for i in members}


def gather_results(local: dict, world: int, dst: int = 0) -> dict | None:
    """Merge the ranks' {member: result} dicts on rank `dst` (None on the
    other ranks).  One object gather through torch.distributed; a single
    process returns its own dict."""
    if world == 1:
        return dict(local)
    import torch.distributed as dist

    rank = dist.get_rank()
    parts = [None] * world if rank == dst else None
    dist.gather_object(local, parts, dst=dst)
    if rank != dst:
        return None
    merged: dict = {}
    for p in parts:
        dup = merged.keys() & p.keys()
        if dup:
            raise RuntimeError(f"members placed on two ranks: {sorted(dup)[:8]}")
        merged.update(p)
    return merged
