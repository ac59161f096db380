// Driver: the reference's Pannotia SSSP mega_kernel (sssp_kernel.cl, included
// by path) run as one work-group of one work-item after vector_init, as in
// pannotia/graph_app/sssp/sssp_gb.cpp:239-310.  Test infrastructure.
#include <vector>
#include "opencl_shim.h"

namespace pnsssp {
#include "sssp/kernel/sssp_kernel.cl"
}

// row/col/data are the CSR the kernel pulls over (the reference passes the
// transposed graph, sssp_gb.cpp:128).
extern "C" int ref_sssp_pannotia(uint32_t V, const uint32_t* row_ptr,
                                 const uint32_t* col, const uint32_t* w,
                                 uint32_t src, int32_t* cost_out) {
  const uint32_t E = row_ptr[V];
  std::vector<int> row(row_ptr, row_ptr + V + 1), c(col, col + E),
      d(w, w + E), x(V), y(V);
  int stop = 0;
  pnsssp::discovery_kernel_ctx ctx;
  shim_single([&] { pnsssp::init_discovery_kernel_ctx(&ctx, 0); });
  shim_ndrange(V, 1, [&] {
    pnsssp::vector_init(x.data(), y.data(), (int)src, (int)V);
  });
  shim_single([&] {
    pnsssp::mega_kernel((int)V, row.data(), c.data(), d.data(), x.data(),
                        y.data(), &stop, &ctx);
  });
  for (uint32_t i = 0; i < V; ++i) cost_out[i] = x[i];
  return 0;
}
