// Host-side helpers for the reference-kernel drivers (test infrastructure):
// build the LonestarGPU 1-based CSR (lonestar/include/graph.h:79-94) and
// relabel a graph so that a chosen vertex becomes vertex 0 (the Lonestar
// kernels hard-code source 0, bfs_port_kernel.cl:133).
#pragma once
#include <stdint.h>
#include <vector>

struct RefCsr {
  uint32_t V = 0, E = 0;
  std::vector<uint32_t> row, col, w;
};

// Swap the ids 0 and s; perm is an involution, so it maps both ways.
static inline RefCsr ref_relabel(uint32_t V, const uint32_t* row_ptr,
                                 const uint32_t* col, const uint32_t* w,
                                 uint32_t s) {
  auto perm = [s](uint32_t x) { return x == 0 ? s : (x == s ? 0 : x); };
  RefCsr g;
  g.V = V;
  g.E = row_ptr[V];
  g.row.resize(V + 1);
  g.col.resize(g.E);
  if (w) g.w.resize(g.E);
  uint32_t o = 0;
  for (uint32_t i = 0; i < V; ++i) {
    g.row[i] = o;
    uint32_t u = perm(i);
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
      g.col[o] = perm(col[e]);
      if (w) g.w[o] = w[e];
      ++o;
    }
  }
  g.row[V] = o;
  return g;
}

// Storage behind a Lonestar `Graph` struct.
struct LonestarStore {
  std::vector<uint32_t> noutgoing, nincoming, srcsrc, psrc, edgessrcdst,
      edgessrcwt;
  uint32_t maxout = 0, maxin = 0;
  void build(const RefCsr& g) {
    noutgoing.assign(g.V, 0);
    nincoming.assign(g.V, 0);
    srcsrc.resize(g.V);
    psrc.assign(g.V + 1, 0);
    edgessrcdst.assign(g.E + 1, 0);  // entry 0 is the null edge
    edgessrcwt.assign(g.E + 1, 0);
    psrc[g.V] = g.E;  // graph.h:83
    for (uint32_t u = 0; u < g.V; ++u) {
      srcsrc[u] = u;
      psrc[u] = g.row[u] + 1;
      noutgoing[u] = g.row[u + 1] - g.row[u];
      for (uint32_t e = g.row[u]; e < g.row[u + 1]; ++e) {
        edgessrcdst[e + 1] = g.col[e];
        edgessrcwt[e + 1] = g.w.empty() ? 1 : g.w[e];
        nincoming[g.col[e]]++;
      }
    }
  }
  template <class G>
  void fill(G& gr, uint32_t V, uint32_t E) {
    gr.nnodes = V;
    gr.nedges = E;
    gr.noutgoing = noutgoing.data();
    gr.nincoming = nincoming.data();
    gr.srcsrc = srcsrc.data();
    gr.psrc = psrc.data();
    gr.edgessrcdst = edgessrcdst.data();
    gr.edgessrcwt = edgessrcwt.data();
    gr.maxOutDegree = &maxout;
    gr.maxInDegree = &maxin;
  }
};
