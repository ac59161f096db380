// Driver: the reference's Pannotia colouring mega_kernel (color_kernel.cl,
// included by path) run as one work-group of one work-item with colours
// initialised to -1 and both stop flags to 0, as in
// pannotia/graph_app/color/color_gb.cpp:145-333.  Test infrastructure.
#include <vector>
#include "opencl_shim.h"

namespace pncolor {
#include "color/kernel/color_kernel.cl"
}

extern "C" int ref_color_pannotia(uint32_t V, const uint32_t* row_ptr,
                                  const uint32_t* col, const float* node_value,
                                  int32_t* color_out) {
  const uint32_t E = row_ptr[V];
  std::vector<int> row(row_ptr, row_ptr + V + 1), c(col, col + E),
      color(V, -1);
  std::vector<float> nv(node_value, node_value + V), mx(V);
  int stop1 = 0, stop2 = 0;
  pncolor::discovery_kernel_ctx ctx;
  shim_single([&] { pncolor::init_discovery_kernel_ctx(&ctx, 0); });
  shim_single([&] {
    pncolor::mega_kernel(row.data(), c.data(), nv.data(), color.data(), &stop1,
                         &stop2, mx.data(), (int)V, (int)E, &ctx);
  });
  for (uint32_t i = 0; i < V; ++i) color_out[i] = color[i];
  return 0;
}
