"""bench.py's end-to-end pipeline: each step's inputs go up into one of two
device buffer sets while the other set's step runs.  Here consecutive steps
get different sources, so a step that read the other set's inputs, or
results read back before their app finished, would show: every step's BFS
levels and SSSP distances must be the oracle's for that step's own
sources."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pipelined_steps_use_their_own_inputs():
    torch = pytest.importorskip("torch")
    import bench
    import oracle
    from gpu_discovery_barrier_gb300 import graphgen as gg

    wl = bench.make_workload(12, 16, None)
    g = wl["g"]
    suite = bench.GpuSuite(wl, ["bfs", "sssp", "mis", "color", "bc", "mst"], 0, "plain")
    h, (d0, d1) = suite.e2e_buffers()
    src_sets = [np.asarray(wl["src"], np.uint32),
                np.asarray(gg.sources(g, bench.NSRC, seed=99), np.uint32)]
    h_alt = dict(h)
    h_alt["src"] = bench.pinned_tensor(torch, src_sets[1])
    hs = [h, h_alt]
    gw = g.with_weights(wl["w"])
    want = [(np.stack([oracle.bfs(g, int(s)) for s in ss]),
             np.stack([oracle.sssp_worklist(gw, int(s)) for s in ss])) for ss in src_sets]
    cs, us = torch.cuda.Stream(), torch.cuda.Stream()
    steps, ev = 4, None
    for k in range(steps):
        d, d_next = (d0, d1) if k % 2 == 0 else (d1, d0)
        _, ev = suite.step_e2e(hs[k % 2], d, cs, ev, d_next if k + 1 < steps else None, us,
                               hs[(k + 1) % 2])
        torch.cuda.synchronize()
        bfs_w, sssp_w = want[k % 2]
        assert np.array_equal(h["bfs"].numpy().view(np.uint32), bfs_w), k
        assert np.array_equal(h["sssp"].numpy().view(np.uint32), sssp_w), k
