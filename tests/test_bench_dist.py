"""bench.py's multi-rank path on CPU: two gloo ranks, barrier and the
max-over-ranks reduction that turns per-rank times into the whole-job time
(replicas only: each rank runs an independent copy of the workload)."""
import os

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank), GDB_BENCH_BACKEND="gloo")
    import bench

    r, w, _ = bench.dist_setup(world)
    bench.barrier(w)
    ms = bench.reduce_max(10.0 + 5.0 * r, w)   # rank 1 is the slow one
    q.put((r, w, ms))
    dist.destroy_process_group()


def test_two_rank_max_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [o[:2] for o in out] == [(0, 2), (1, 2)]
    assert all(o[2] == 15.0 for o in out)
