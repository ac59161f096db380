// Driver: the reference's Pannotia MIS mega_kernel (mis_kernel.cl, included
// by path) run as one work-group of one work-item after the init kernel, as
// in pannotia/graph_app/mis/mis_gb.cpp.  Test infrastructure.
#include <vector>
#include "opencl_shim.h"

namespace pnmis {
#include "mis/kernel/mis_kernel.cl"
}

extern "C" int ref_mis_pannotia(uint32_t V, const uint32_t* row_ptr,
                                const uint32_t* col, const float* node_value,
                                int32_t* s_out) {
  const uint32_t E = row_ptr[V];
  std::vector<int> row(row_ptr, row_ptr + V + 1), c(col, col + E), s(V),
      ca(V), cu(V);
  std::vector<float> nv(node_value, node_value + V), mn(V);
  int stop = 0;  // mis_gb.cpp:295-298
  pnmis::discovery_kernel_ctx ctx;
  shim_single([&] { pnmis::init_discovery_kernel_ctx(&ctx, 0); });
  shim_ndrange(V, 1, [&] {
    pnmis::init(s.data(), ca.data(), cu.data(), (int)V, (int)E);
  });
  shim_single([&] {
    pnmis::mega_kernel(row.data(), c.data(), nv.data(), s.data(), ca.data(),
                       cu.data(), mn.data(), &stop, (int)V, (int)E, &ctx);
  });
  for (uint32_t i = 0; i < V; ++i) s_out[i] = s[i];
  return 0;
}
