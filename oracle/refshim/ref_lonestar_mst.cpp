// Driver: the reference's LonestarGPU Boruvka MST (mst_port_kernel.cl,
// included by path).  The round loop is the host loop of
// lonestar/apps/mst/mst_port.cpp:202-312: dinit, dfindelemin, dfindelemin2
// and verify_min_elem as sequential NDRange loops, then the persistent
// dfindcompmintwo (one work-group of one work-item) until `repeat` stays 0;
// rounds continue while the component count changes.  Test infrastructure.
#include <vector>
#include "opencl_shim.h"
#include "ref_graph.h"

namespace lsmst {
#include "mst_port_kernel.cl"
}

extern "C" int ref_mst_lonestar(uint32_t V, const uint32_t* row_ptr,
                                const uint32_t* col, const uint32_t* w,
                                uint32_t* weight_out, uint32_t* components_out,
                                uint32_t* edges_out) {
  RefCsr g;
  g.V = V;
  g.E = row_ptr[V];
  g.row.assign(row_ptr, row_ptr + V + 1);
  g.col.assign(col, col + g.E);
  g.w.assign(w, w + g.E);
  LonestarStore st;
  st.build(g);
  lsmst::Graph gr;
  st.fill(gr, g.V, g.E);

  std::vector<uint32_t> eleminwts(V), minwtcomponent(V), partners(V),
      phores(V), goahead(V), ncomp(1), complen(V), ele2comp(V);
  std::vector<int> pinn(V);
  uint32_t mstwt = 0;
  int repeat = 0, count = 0;
  lsmst::ComponentSpace cs;
  shim_ndrange(((V + 255) / 256) * 256, 256, [&] {
    lsmst::init_compspace(&cs, ncomp.data(), complen.data(), ele2comp.data(),
                          V);
  });
  lsmst::discovery_kernel_ctx ctx;
  shim_single([&] { lsmst::init_discovery_kernel_ctx(&ctx, 0); });

  unsigned prev, cur = V;
  const size_t gs = ((V + 127) / 128) * 128;
#define MST_ARGS                                                           \
  &mstwt, &gr, &cs, eleminwts.data(), minwtcomponent.data(), partners.data(), \
      phores.data(), pinn.data(), goahead.data()
  do {
    prev = cur;
    shim_ndrange(gs, 128, [&] { lsmst::dinit(MST_ARGS); });
    shim_ndrange(gs, 128, [&] { lsmst::dfindelemin(MST_ARGS); });
    shim_ndrange(gs, 128, [&] { lsmst::dfindelemin2(MST_ARGS); });
    shim_ndrange(gs, 128, [&] { lsmst::verify_min_elem(MST_ARGS); });
    do {
      repeat = 0;
      shim_single([&] { lsmst::dfindcompmintwo(MST_ARGS, &repeat, &count, &ctx); });
    } while (repeat);
    cur = ncomp[0];
  } while (cur != prev);
#undef MST_ARGS
  *weight_out = mstwt;
  *components_out = cur;
  *edges_out = (uint32_t)count;
  return 0;
}
