// Driver: the reference's LonestarGPU Delaunay mesh refinement kernels
// (dmr_port_kernel.cl with dmr_common.cl, included by path) with the host
// sequence of lonestar/apps/dmr/dmr_port.cpp:160-316: neighbours as
// find_neighbours_cpu (dmr.h:55-104, restated here: dmr.h also holds the
// OpenCL host set-up), check_triangles from element 0, then refine and
// check_triangles from the previous element count until no bad triangle is
// left.  refine runs as one work-group of one work-item, so every item of a
// round is processed in order and none conflicts; check_triangles runs one
// work-item per element, so its pushes come in element order.  Both
// worklists hold maxnelements entries (the reference sizes them by the
// initial element count, and its wl_push drops items past that).
// rsqrt(v) is read as 1 / sqrt(v).  Test infrastructure.
#include <cmath>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "opencl_shim.h"

namespace lsdmr {
#define cl_khr_fp64 1
struct uint3 {
  uint x, y, z;
};
static inline double rsqrt(double v) { return 1.0 / std::sqrt(v); }
using std::cos;
#define global  // dmr_common.cl:473 spells the qualifier without underscores
#include "dmr_port_kernel.cl"
#undef global
#undef cl_khr_fp64
}  // namespace lsdmr

namespace {

void add_neighbour_cpu(lsdmr::uint3& n, uint e) {
  if (n.x == e || n.y == e || n.z == e) return;
  if (n.x == INVALIDID) { n.x = e; return; }
  if (n.y == INVALIDID) { n.y = e; return; }
  if (n.z == INVALIDID) { n.z = e; return; }
}

}  // namespace

extern "C" int ref_dmr_lonestar(const double* x0, const double* y0, uint32_t nnodes,
                                const uint32_t* el0, uint32_t nelements, uint32_t maxfactor,
                                double* x_out, double* y_out, uint32_t* el_out, uint32_t* nb_out,
                                uint8_t* isdel_out, uint32_t* counts) {
  const uint32_t maxn = (maxfactor / 2) * nnodes, maxe = maxfactor * nelements;
  std::vector<double> nodex(maxn), nodey(maxn);
  std::vector<lsdmr::uint3> elements(maxe), neighbours(maxe);
  std::vector<int> isdel(maxe, 0), isbad(maxe, 0), owners(maxe, 0);
  std::memcpy(nodex.data(), x0, sizeof(double) * nnodes);
  std::memcpy(nodey.data(), y0, sizeof(double) * nnodes);
  for (uint32_t e = 0; e < nelements; ++e)
    elements[e] = {el0[3 * e], el0[3 * e + 1], el0[3 * e + 2]};
  // find_neighbours_cpu
  std::map<std::pair<uint, uint>, uint> edge_map;
  for (uint32_t e = 0; e < nelements; ++e) {
    neighbours[e] = {INVALIDID, INVALIDID, INVALIDID};
    uint n[3] = {elements[e].x, elements[e].y, elements[e].z};
    if (n[0] > n[1]) std::swap(n[0], n[1]);
    if (n[1] > n[2]) std::swap(n[1], n[2]);
    if (n[0] > n[1]) std::swap(n[0], n[1]);
    const std::pair<uint, uint> edges[3] = {{n[0], n[1]}, {n[1], n[2]}, {n[0], n[2]}};
    const int maxk = elements[e].z == INVALIDID ? 1 : 3;
    for (int i = 0; i < maxk; ++i) {
      auto it = edge_map.find(edges[i]);
      if (it == edge_map.end()) {
        edge_map[edges[i]] = e;
      } else {
        add_neighbour_cpu(neighbours[it->second], e);
        add_neighbour_cpu(neighbours[e], it->second);
        edge_map.erase(it);
      }
    }
  }
  lsdmr::Mesh mesh;
  uint ntri = 0;
  for (uint32_t e = 0; e < nelements; ++e) ntri += elements[e].z != INVALIDID;
  shim_single([&] {
    lsdmr::init_mesh(&mesh, nodex.data(), nodey.data(), elements.data(), neighbours.data(),
                     isdel.data(), isbad.data(), owners.data(), maxe, maxn, ntri, nnodes,
                     nelements - ntri, nelements);
  });
  uint d_nnodes = nnodes, d_nelements = nelements, nbad = 0;
  std::vector<int> w1(maxe), w2(maxe);
  int n1 = (int)maxe, n2 = (int)maxe, i1 = 0, i2 = 0;
  lsdmr::CL_Worklist2 inwl{w1.data(), &n1, &i1}, outwl{w2.data(), &n2, &i2};
  lsdmr::discovery_kernel_ctx ctx;
  shim_single([&] { lsdmr::init_discovery_kernel_ctx(&ctx, 0); });

  auto check = [&](lsdmr::CL_Worklist2* wl, int start) {
    const uint32_t n = mesh.nelements > (uint)start ? mesh.nelements - start : 1;
    shim_ndrange(n, 1, [&] { lsdmr::check_triangles(&mesh, &nbad, wl, start); });
  };
  check(&inwl, 0);
  lsdmr::CL_Worklist2* in = &inwl;
  lsdmr::CL_Worklist2* out = &outwl;
  uint32_t rounds = 0;
  while (*in->dindex) {
    if (++rounds > 100000) return -4;
    const int last = (int)mesh.nelements;
    shim_single([&] { lsdmr::refine(&mesh, &d_nnodes, &d_nelements, in, out, &ctx); });
    if (d_nelements > maxe || d_nnodes > maxn) return -3;
    *in->dindex = 0;  // wl_reset of the consumed list
    check(out, last);
    if (*out->dindex > (int)maxe) return -3;
    std::swap(in, out);
  }
  const uint32_t nn = mesh.nnodes, ne = mesh.nelements;
  std::memcpy(x_out, nodex.data(), sizeof(double) * nn);
  std::memcpy(y_out, nodey.data(), sizeof(double) * nn);
  for (uint32_t e = 0; e < ne; ++e) {
    el_out[3 * e] = elements[e].x;
    el_out[3 * e + 1] = elements[e].y;
    el_out[3 * e + 2] = elements[e].z;
    nb_out[3 * e] = neighbours[e].x;
    nb_out[3 * e + 1] = neighbours[e].y;
    nb_out[3 * e + 2] = neighbours[e].z;
    isdel_out[e] = (uint8_t)(isdel[e] != 0);
  }
  counts[0] = nn;
  counts[1] = ne;
  counts[2] = rounds;
  counts[3] = rounds;
  counts[4] = 0;
  return 0;
}
