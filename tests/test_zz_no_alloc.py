"""The allocation-free BFS entry point (gdb_bfs_noalloc) against gdb_bfs.

gdb_bfs_noalloc exists for callers that cannot allocate device memory (a
host whose own pool owns the GPU's memory, a plug-in that must not trigger
cudaMalloc's device synchronisation): it takes plain device pointers and
keeps its scratch in a fixed array inside the library.  Its levels must be
bit-identical to the regular entry point's, on two calls in a row (the
second call reuses the array the first one left behind).  This file is
collected last so a failure here cannot hide the other tests' results.
"""
import numpy as np
import pytest

from gpu_discovery_barrier_gb300 import gdb, graphgen as gg

pytestmark = pytest.mark.gpu


def _device_graph(torch, g):
    dev = torch.device("cuda", 0)
    row = torch.from_numpy(g.row_ptr.view(np.int32)).to(dev)
    col = torch.from_numpy(g.col.view(np.int32) if g.E else np.zeros(1, np.int32)).to(dev)
    return row, col


@pytest.mark.parametrize("make", [lambda: gg.rmat(1 << 16, 16, seed=21), lambda: gg.grid(300, 200)],
                         ids=["rmat16", "grid300x200"])
def test_noalloc_matches_bfs_twice(make):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = make()
    srcs = [int(s) for s in gg.sources(g, 2, seed=5)]
    with gdb.Ctx() as c:
        G = c.graph(g.row_ptr, g.col)
        want = [c.bfs(G, s) for s in srcs]
    row, col = _device_graph(torch, g)
    out = torch.empty(g.V, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for s, w in zip(srcs, want):
        out.fill_(-7)  # stale contents must not leak into the answer
        torch.cuda.synchronize()
        gdb.bfs_noalloc(row.data_ptr(), col.data_ptr(), g.V, g.E, s, out.data_ptr(), stream)
        got = out.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, w), s


def test_noalloc_rejects_oversized_graphs():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    with pytest.raises(gdb.GdbError) as e:
        gdb.bfs_noalloc(1, 1, gdb.NOALLOC_MAX_VERTICES + 1, 1, 0, 1, 0)
    assert e.value.status == -1
