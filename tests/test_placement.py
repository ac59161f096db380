"""Graph -> GPU placement of the batched and serving forms (host logic, CPU).

Whole graphs go to one rank each, balanced by arcs; every rank derives the
same placement from the batch's sizes, builds only its own members, and the
results are gathered on rank 0.  The two-rank test runs the real
torch.distributed path over gloo: each rank computes the oracle's BFS levels
for its members, rank 0 gathers them and checks that every member arrives
exactly once and equals the single-process answer.
"""
import os

import numpy as np
import pytest

from gpu_discovery_barrier_gb300 import graphgen as gg, placement


def test_place_covers_every_member_once_and_balances():
    rng = np.random.default_rng(3)
    arcs = rng.integers(1, 10_000, 200)
    for world in (1, 2, 3, 8):
        p = placement.place(arcs, world)
        flat = sorted(i for r in p for i in r)
        assert flat == list(range(len(arcs)))
        loads = [int(arcs[r].sum()) if r else 0 for r in p]
        # longest-processing-time first: no rank exceeds the mean by more
        # than the largest member
        assert max(loads) <= arcs.sum() / world + arcs.max()
        assert p == placement.place(arcs, world)  # deterministic
    assert placement.place(arcs, 1) == [list(range(len(arcs)))]


def test_place_more_ranks_than_members():
    p = placement.place([5, 3], 4)
    assert sorted(i for r in p for i in r) == [0, 1]
    assert sum(1 for r in p if not r) == 2
    assert placement.owner_of(p) == {0: 0, 1: 1}


def test_subset_members_equal_the_full_batch():
    full = gg.mixed_batch(9, 100, 4000, seed=7)
    spec = gg.mixed_batch_spec(9, 100, 4000, seed=7)
    part = gg.mixed_batch(9, 100, 4000, seed=7, members=[8, 3, 0])
    for g, i in zip(part, [8, 3, 0]):
        assert np.array_equal(g.row_ptr, full[i].row_ptr)
        assert np.array_equal(g.col, full[i].col) and np.array_equal(g.w, full[i].w)
        assert g.meta["source"] == full[i].meta["source"]
        assert g.V == spec[i]["V"]
        if spec[i]["kind"] == "grid":
            assert g.E == spec[i]["arcs"]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank), GDB_BENCH_BACKEND="gloo")
    import torch.distributed as dist

    import bench
    import oracle

    try:
        r, w, _ = bench.dist_setup(world)
        mine = bench.my_members(12, r, w, seed=5)
        members = gg.mixed_batch(12, 50, 3000, seed=5, members=mine)
        local = {g.meta["member"]: oracle.bfs(g, g.meta["source"]).tolist() for g in members}
        units = bench.reduce_sum(float(sum(g.E for g in members)), w)
        merged = placement.gather_results(local, w)
        out = None
        if r == 0:
            full = gg.mixed_batch(12, 50, 3000, seed=5)
            want = {i: oracle.bfs(g, g.meta["source"]).tolist() for i, g in enumerate(full)}
            out = (sorted(merged) == list(range(12)), merged == want,
                   units == float(sum(g.E for g in full)), sorted(len(x) for x in [mine]))
        q.put((r, out))
        dist.destroy_process_group()
    except Exception as e:  # report instead of hanging the parent
        q.put((rank, repr(e)))


def test_two_rank_placement_and_gather():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp  # noqa: F401

    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = 31500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert out[1] is None, out
    covered, equal, units_ok, _ = out[0]
    assert covered and equal and units_ok, out
