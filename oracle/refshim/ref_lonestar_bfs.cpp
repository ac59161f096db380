// Driver: the reference's LonestarGPU BFS kernels (bfs_port_kernel.cl,
// included by path) run as one work-group of one work-item, with the host
// sequence of lonestar/apps/bfs/bfs_port.cpp:62-194.  Test infrastructure.
#include "opencl_shim.h"
#include "ref_graph.h"

namespace lsbfs {
#include "bfs_port_kernel.cl"
}

extern "C" int ref_bfs_lonestar(uint32_t V, const uint32_t* row_ptr,
                                const uint32_t* col, uint32_t src,
                                uint32_t* dist_out) {
  if (src >= V) return -1;
  RefCsr g = ref_relabel(V, row_ptr, col, nullptr, src);
  LonestarStore st;
  st.build(g);
  lsbfs::Graph gr;
  st.fill(gr, g.V, g.E);

  std::vector<uint32_t> dist(V);
  uint32_t gerrno = 0;
  // worklists of capacity nedges (bfs_port.cpp:135-136); one work-item never
  // pushes a vertex twice, so V + 1 slots also suffice
  int cap = (int)((g.E > V ? g.E : V) + 1);
  std::vector<int> w1(cap), w2(cap);
  int n1 = cap, n2 = cap, i1 = 0, i2 = 0;
  lsbfs::CL_Worklist2 wl1{w1.data(), &n1, &i1}, wl2{w2.data(), &n2, &i2};
  lsbfs::discovery_kernel_ctx ctx;

  shim_ndrange(V, 1, [&] { lsbfs::initialize(dist.data(), V); });
  dist[0] = 0;  // bfs_port.cpp:112-121
  shim_single([&] { lsbfs::init_discovery_kernel_ctx(&ctx, 0); });
  shim_single([&] {
    lsbfs::drelax2(dist.data(), &gr, &gerrno, &wl1, &wl2, 0, &ctx);
  });
  shim_single([&] {
    lsbfs::drelax2(dist.data(), &gr, &gerrno, &wl1, &wl2, 1, &ctx);
  });
  for (uint32_t i = 0; i < V; ++i) {
    uint32_t old = i == 0 ? src : (i == src ? 0 : i);
    dist_out[old] = dist[i];
  }
  return (int)gerrno;
}
