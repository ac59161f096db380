// Driver: the reference's LonestarGPU worklist SSSP (sssp_port_kernel.cl,
// included by path) run as one work-group of one work-item, with the host
// sequence of lonestar/apps/sssp/sssp_port.cpp.  Test infrastructure.
#include "opencl_shim.h"
#include "ref_graph.h"

namespace lssssp {
#include "sssp_port_kernel.cl"
}

extern "C" int ref_sssp_lonestar(uint32_t V, const uint32_t* row_ptr,
                                 const uint32_t* col, const uint32_t* w,
                                 uint32_t src, uint32_t* dist_out) {
  if (src >= V) return -1;
  RefCsr g = ref_relabel(V, row_ptr, col, w, src);
  LonestarStore st;
  st.build(g);
  lssssp::Graph gr;
  st.fill(gr, g.V, g.E);

  std::vector<uint32_t> dist(V);
  // A vertex may be pushed once per improvement; bound the queue by the
  // number of arcs plus one, which a single work-item cannot exceed within
  // one superstep.
  int cap = (int)(g.E + V + 1);
  std::vector<int> w1(cap), w2(cap);
  int n1 = cap, n2 = cap, i1 = 0, i2 = 0;
  lssssp::CL_Worklist2 wl1{w1.data(), &n1, &i1}, wl2{w2.data(), &n2, &i2};
  lssssp::discovery_kernel_ctx ctx;

  shim_ndrange(V, 1, [&] { lssssp::initialize(dist.data(), V); });
  dist[0] = 0;
  shim_single([&] { lssssp::init_discovery_kernel_ctx(&ctx, 0); });
  shim_single([&] { lssssp::drelax2(dist.data(), &gr, &wl1, &wl2, 0, &ctx); });
  shim_single([&] { lssssp::drelax2(dist.data(), &gr, &wl1, &wl2, 1, &ctx); });
  for (uint32_t i = 0; i < V; ++i) {
    uint32_t old = i == 0 ? src : (i == src ? 0 : i);
    dist_out[old] = dist[i];
  }
  return 0;
}
