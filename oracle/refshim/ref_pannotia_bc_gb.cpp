// Driver: the reference's Pannotia mega_bc_kernel (bc_kernel.cl with GB_VAR,
// included by path) run as one work-group of one work-item: whole-graph BC
// over every source, after clean_bc and zeroed stop flags
// (pannotia/graph_app/bc/bc_gb.cpp:315-344).  The V*V dependency array `p`
// is zeroed by the kernel and never read, so this driver is for small
// graphs only.  Test infrastructure.
#include <vector>
#include "opencl_shim.h"

#define GB_VAR 1
namespace pnbcgb {
#include "bc/kernel/bc_kernel.cl"
}

extern "C" int ref_bc_pannotia_gb(uint32_t V, const uint32_t* row_ptr,
                                  const uint32_t* col, const uint32_t* trow,
                                  const uint32_t* tcol, float* bc_out) {
  const uint32_t E = row_ptr[V];
  if ((uint64_t)V * V > (1ull << 26)) return -1;
  std::vector<int> row(row_ptr, row_ptr + V + 1), c(col, col + E),
      rt(trow, trow + V + 1), ct(tcol, tcol + E), dist(V), p((size_t)V * V);
  std::vector<float> rho(V), sigma(V), bc(V);
  int s1 = 0, s2 = 0, s3 = 0, gd = 0;
  pnbcgb::discovery_kernel_ctx ctx;
  shim_single([&] { pnbcgb::init_discovery_kernel_ctx(&ctx, 0); });
  shim_ndrange(V, 1, [&] { pnbcgb::clean_bc(bc.data(), (int)V); });
  shim_single([&] {
    pnbcgb::mega_bc_kernel(row.data(), c.data(), rt.data(), ct.data(),
                           dist.data(), rho.data(), sigma.data(), p.data(),
                           &s1, &s2, &s3, &gd, bc.data(), (int)V, (int)E, &ctx);
  });
  for (uint32_t i = 0; i < V; ++i) bc_out[i] = bc[i];
  return 0;
}
