// Driver: the reference's Pannotia multi-kernel BC (bc_kernel.cl without
// GB_VAR, included by path): clean_1d_array, then bfs_kernel launches until
// the stop flag stays 0, then backtrack_kernel from the deepest level,
// following the host loop of pannotia/graph_app/bc/bc.cpp:322-420 but over a
// given list of sources.  Each NDRange kernel runs as a sequential loop over
// its global ids.  clean_2d_array is skipped: `p` is zeroed and never read.
// Test infrastructure.
#include <vector>
#include "opencl_shim.h"

namespace pnbcmk {
#include "bc/kernel/bc_kernel.cl"
}

extern "C" int ref_bc_pannotia_sources(uint32_t V, const uint32_t* row_ptr,
                                       const uint32_t* col,
                                       const uint32_t* trow,
                                       const uint32_t* tcol,
                                       const uint32_t* sources, uint32_t nsrc,
                                       float* bc_out) {
  const uint32_t E = row_ptr[V];
  std::vector<int> row(row_ptr, row_ptr + V + 1), c(col, col + E),
      rt(trow, trow + V + 1), ct(tcol, tcol + E), d(V), p(1);
  std::vector<float> rho(V), sigma(V), bc(V);
  int stop = 0;
  shim_ndrange(V, 1, [&] { pnbcmk::clean_bc(bc.data(), (int)V); });
  for (uint32_t k = 0; k < nsrc; ++k) {
    int s = (int)sources[k];
    shim_ndrange(V, 1, [&] {
      pnbcmk::clean_1d_array(s, d.data(), sigma.data(), rho.data(), (int)V);
    });
    int dist = 0;
    do {
      stop = 0;
      shim_ndrange(V, 1, [&] {
        pnbcmk::bfs_kernel(row.data(), c.data(), d.data(), rho.data(),
                           p.data(), &stop, (int)V, (int)E, dist);
      });
      dist++;
    } while (stop);
    while (dist) {
      shim_ndrange(V, 1, [&] {
        pnbcmk::backtrack_kernel(rt.data(), ct.data(), d.data(), rho.data(),
                                 sigma.data(), p.data(), (int)V, (int)E, dist,
                                 s, bc.data());
      });
      dist--;
    }
  }
  for (uint32_t i = 0; i < V; ++i) bc_out[i] = bc[i];
  return 0;
}
