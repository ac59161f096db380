"""GPU tests of the discovery protocol and the barriers.

Every wait in the device code has a deadline; the timeout test stalls the
XF master through the library's test hook (a flag nothing releases) and
checks that the kernel ends with GDB_ERR_TIMEOUT and the context stays
usable -- no trap, no fault, no hang.
"""
import pytest

from gpu_discovery_barrier_gb300 import gdb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lock", [gdb.LOCK_TICKET, gdb.LOCK_SPIN, gdb.LOCK_FREE])
def test_occupancy_test_discovers_coresident(lock):
    with gdb.Ctx(lock=lock) as c:
        fit = c.api_occupancy(256)
        assert fit > 0
        # exactly the API occupancy: every CTA can be co-resident
        n = c.occupancy_test(fit, 256)
        assert 1 <= n <= fit
        # over-subscribed like the reference (1000 + fit CTAs): only
        # co-resident CTAs take part and the barrier still completes
        n2 = c.occupancy_test(fit + 1000, 256)
        assert 1 <= n2 <= fit
        assert c.number_of_participating_groups() == n2


@pytest.mark.parametrize("lock", [gdb.LOCK_TICKET, gdb.LOCK_FREE])
def test_protocol_self_resets(lock):
    """The last CTA re-arms the context, so launches need no re-init
    (discovery.cl:32-36 / reset_kernel_context)."""
    with gdb.Ctx(lock=lock) as c:
        fit = c.api_occupancy(128)
        for _ in range(3):
            ns = c.time_protocol(fit, 128)
            assert ns > 0
            assert 1 <= c.number_of_participating_groups() <= fit


def test_skip_refuses_oversubscription():
    with gdb.Ctx() as c:
        fit = c.api_occupancy(256)
        c.init_discovery_kernel_ctx(skip=1)
        with pytest.raises(gdb.GdbError) as e:
            c.occupancy_test(fit + 1, 256)
        assert e.value.status == -6
        assert c.occupancy_test(fit, 256) == fit
        c.init_discovery_kernel_ctx()


@pytest.mark.parametrize("xf_release", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("kind", [gdb.BARRIER_XF, gdb.BARRIER_XF_FIXED, gdb.BARRIER_GRID_SYNC,
                                  gdb.BARRIER_RELAUNCH, gdb.BARRIER_RELAUNCH_GRAPH])
def test_barrier_bench(kind, xf_release):
    with gdb.Ctx(xf_release=xf_release) as c:
        ns, groups = c.barrier_bench(kind, 256, 200)
        assert ns > 0 and groups >= 1


def test_release_modes_switch_in_one_context():
    """Switching the XF release form must not leave stale arrivals."""
    import numpy as np

    import oracle
    from gpu_discovery_barrier_gb300 import graphgen as gg

    g = gg.rmat(1 << 12, 8, seed=3)
    with gdb.Ctx() as c:
        G = c.graph(g.row_ptr, g.col)
        want = oracle.bfs(g, 1)
        for rel in (1, 0, 2, 3, 1, 4, 3, 2, 0, 3, 4):
            c.set_options(xf_release=rel)
            assert np.array_equal(c.bfs(G, 1), want)
            c.barrier_bench(gdb.BARRIER_XF, 256, 50)


@pytest.mark.parametrize("xf_release", [0, 1, 2, 3, 4])
def test_timeout_reports_and_recovers(xf_release):
    with gdb.Ctx(timeout_ns=50_000_000, xf_release=xf_release) as c:
        c.debug_stall_master(3)
        with pytest.raises(gdb.GdbError) as e:
            c.barrier_bench(gdb.BARRIER_XF, 256, 20)
        assert e.value.status == -4
        c.debug_stall_master(-1)
        ns, groups = c.barrier_bench(gdb.BARRIER_XF, 256, 20)
        assert ns > 0 and groups >= 1


@pytest.mark.parametrize("xf_release", [2, 3, 4])
@pytest.mark.parametrize("ctas", [1, 2, 17, 152, 0])
def test_counting_barrier_group_sizes(ctas, xf_release):
    """Arrival counts for every participant count, including a lone master
    and counts that do not divide by the 16 groups; repeated launches reuse
    the context (combining: counts zeroed at the end of each; flat: the
    next launch starts from the count the last one reached)."""
    with gdb.Ctx(xf_release=xf_release, max_ctas=ctas) as c:
        for _ in range(3):
            ns, groups = c.barrier_bench(gdb.BARRIER_XF, 256, 300)
            assert ns > 0 and groups >= 1
            if ctas:
                assert groups <= ctas


@pytest.mark.parametrize("xf_release", [0, 1, 2, 3, 4])
def test_all_apps_on_every_xf_form(xf_release):
    import numpy as np

    import oracle
    from gpu_discovery_barrier_gb300 import graphgen as gg

    g = gg.rmat(1 << 12, 12, seed=8)
    w = gg.uniform_weights(g, 1, 255, seed=2)
    uw = gg.unique_weights(g, seed=3)
    prio = gg.priorities(g.V, seed=4)
    gw = g.with_weights(w)
    with gdb.Ctx(xf_release=xf_release) as c:
        G = c.graph(g.row_ptr, g.col, w)
        for _ in range(2):
            assert np.array_equal(c.bfs(G, 3), oracle.bfs(g, 3))
            assert np.array_equal(c.sssp(G, 3), oracle.sssp_worklist(gw, 3))
            assert np.array_equal(c.sssp_jacobi(G, 3), oracle.sssp_jacobi(gw, 3, literal=True))
            assert np.array_equal(c.mis(G, prio), oracle.mis(g, prio)[0])
            assert np.array_equal(c.color(G, prio), oracle.color(g, prio)[0])
            got = c.bc(G, [0, 5]).astype(np.float64)
            want = oracle.bc_f64(g, [0, 5])
            assert np.allclose(got, want, rtol=1e-4, atol=1e-3)
        # the learned schedule's decision runs as a hook inside every barrier
        from gpu_discovery_barrier_gb300 import selector

        p = selector.load()
        if p is not None:
            c.selector_set(p)
            c.set_options(schedule=gdb.SCHED_LEARNED)
            assert np.array_equal(c.bfs(G, 3), oracle.bfs(g, 3))
            c.set_options(schedule=gdb.SCHED_PLAIN)
        G.set_weights(uw)
        assert c.mst(G)["weight64"] == oracle.mst(g.with_weights(uw))["weight64"]
