/* CPU oracle for the discovery-barrier graph path -- TEST INFRASTRUCTURE.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
 * this file, as the checker or as the timed CPU baseline; the product
 * library never links it.  Each function restates one reference kernel in
 * plain serial C and cites the reference file:line it follows.  Parity of
 * these restatements is pinned against the reference's own OpenCL C,
 * compiled as C++ through oracle/refshim, by tests/test_oracle_golden.py.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ BFS */

/* Lonestar worklist BFS (lonestar/apps/bfs/kernel/bfs_port_kernel.cl:146-192,
 * processedge2 bfs_common.cl:73-90): dist[src] = 0, every vertex first
 * reached in superstep `iteration` (1, 2, ...) gets dist = iteration, the
 * others keep MYINFINITY.  A FIFO queue visits vertices in the same level
 * order, so the levels are identical. */
int orc_bfs(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
            uint32_t src, uint32_t* dist) {
  if (src >= V) return -1;
  uint32_t* q = (uint32_t*)malloc(sizeof(uint32_t) * (V ? V : 1));
  if (!q) return -2;
  for (uint32_t i = 0; i < V; ++i) dist[i] = ORC_LONESTAR_INF;
  uint32_t head = 0, tail = 0;
  dist[src] = 0;
  q[tail++] = src;
  while (head < tail) {
    uint32_t u = q[head++];
    uint32_t nd = dist[u] + 1;
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
      uint32_t v = col[e];
      if (v >= V) continue; /* bfs_common.cl:80 */
      if (dist[v] == ORC_LONESTAR_INF) {
        dist[v] = nd;
        q[tail++] = v;
      }
    }
  }
  free(q);
  return 0;
}

/* ------------------------------------------------------------- heaps */

typedef struct {
  uint64_t* key; /* (dist << 32) | vertex */
  uint32_t n, cap;
} heap_t;

static int heap_push(heap_t* h, uint64_t k) {
  if (h->n == h->cap) {
    uint32_t nc = h->cap ? h->cap * 2 : 1024;
    uint64_t* nk = (uint64_t*)realloc(h->key, sizeof(uint64_t) * nc);
    if (!nk) return -1;
    h->key = nk;
    h->cap = nc;
  }
  uint32_t i = h->n++;
  while (i > 0) {
    uint32_t p = (i - 1) / 2;
    if (h->key[p] <= k) break;
    h->key[i] = h->key[p];
    i = p;
  }
  h->key[i] = k;
  return 0;
}

static uint64_t heap_pop(heap_t* h) {
  uint64_t top = h->key[0];
  uint64_t last = h->key[--h->n];
  uint32_t i = 0;
  for (;;) {
    uint32_t l = 2 * i + 1;
    if (l >= h->n) break;
    uint32_t m = (l + 1 < h->n && h->key[l + 1] < h->key[l]) ? l + 1 : l;
    if (h->key[m] >= last) break;
    h->key[i] = h->key[m];
    i = m;
  }
  if (h->n) h->key[i] = last;
  return top;
}

/* Shortest distances with a start value `inf` for unreached vertices; an
 * arc is relaxed only when the new distance is below the current one, so a
 * vertex whose shortest distance is >= inf keeps inf -- the fixed point of
 * both reference SSSP kernels. */
static int dijkstra_u32(uint32_t V, const uint32_t* row_ptr,
                        const uint32_t* col, const uint32_t* w, uint32_t src,
                        uint32_t inf, uint32_t skip_w_at_least,
                        uint32_t* dist) {
  if (src >= V) return -1;
  heap_t h = {0, 0, 0};
  for (uint32_t i = 0; i < V; ++i) dist[i] = inf;
  dist[src] = 0;
  if (heap_push(&h, (uint64_t)src)) return -2;
  while (h.n) {
    uint64_t k = heap_pop(&h);
    uint32_t u = (uint32_t)k, du = (uint32_t)(k >> 32);
    if (du != dist[u]) continue;
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
      uint32_t v = col[e];
      uint32_t wt = w ? w[e] : 1;
      if (v >= V || wt >= skip_w_at_least) continue;
      uint64_t nd = (uint64_t)du + wt;
      if (nd < dist[v]) {
        dist[v] = (uint32_t)nd;
        if (heap_push(&h, (nd << 32) | v)) { free(h.key); return -2; }
      }
    }
  }
  free(h.key);
  return 0;
}

/* Lonestar worklist SSSP (lonestar/apps/sssp/kernel/sssp_port_kernel.cl:152-197,
 * processedge2 sssp_common.cl:58-81): label-correcting relaxation with
 * atomic_min; arcs of weight >= MYINFINITY are skipped (sssp_common.cl:70).
 * Its fixed point is the shortest-distance vector computed here. */
int orc_sssp_worklist(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                      const uint32_t* w, uint32_t src, uint32_t* dist) {
  return dijkstra_u32(V, row_ptr, col, w, src, ORC_LONESTAR_INF,
                      ORC_LONESTAR_INF, dist);
}

/* Pannotia Jacobi SSSP, literal restatement of mega_kernel
 * (pannotia/graph_app/sssp/kernel/sssp_kernel.cl:170-244) after vector_init
 * (:111-132): per iteration x = y; y[v] = min(x[v], min_j data[j] + x[col[j]])
 * over the CSR given (the reference passes the transposed graph,
 * sssp_gb.cpp:128); stop when y == x or after num_rows - 1 iterations. */
int orc_sssp_jacobi(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                    const uint32_t* w, uint32_t src, int32_t* cost,
                    uint32_t* iterations) {
  if (src >= V) return -1;
  int32_t* x = cost;
  int32_t* y = (int32_t*)malloc(sizeof(int32_t) * V);
  if (!y) return -2;
  for (uint32_t i = 0; i < V; ++i) x[i] = y[i] = (i == src) ? 0 : ORC_PANNOTIA_BIG;
  uint32_t it = 0;
  for (uint32_t k = 1; k < V; ++k) {
    memcpy(x, y, sizeof(int32_t) * V);
    ++it;
    int stop = 0;
    for (uint32_t v = 0; v < V; ++v) {
      int64_t m = x[v];
      for (uint32_t j = row_ptr[v]; j < row_ptr[v + 1]; ++j) {
        int64_t c = (int64_t)(int32_t)w[j] + x[col[j]];
        if (c < m) m = c;
      }
      y[v] = (int32_t)m;
    }
    for (uint32_t v = 0; v < V; ++v)
      if (y[v] != x[v]) stop = 1;
    if (!stop) break;
  }
  /* The host reads x (vector_d1, sssp_gb.cpp:310): equal to y once
   * converged, but one iteration behind when the k < num_rows cap ends the
   * loop first (a path of V vertices then leaves its far end at BIG_NUM). */
  free(y);
  if (iterations) *iterations = it;
  return 0;
}

/* Same fixed point as orc_sssp_jacobi (cost = min(BIG_NUM, distance)),
 * computed with Dijkstra so it finishes on large graphs.  Equal to the
 * Jacobi result whenever the iteration converges before the num_rows - 1
 * cap, i.e. when no shortest path needs V - 1 arcs. */
int orc_sssp_dijkstra_int(uint32_t V, const uint32_t* row_ptr,
                          const uint32_t* col, const uint32_t* w, uint32_t src,
                          int32_t* cost) {
  return dijkstra_u32(V, row_ptr, col, w, src, (uint32_t)ORC_PANNOTIA_BIG,
                      0xFFFFFFFFu, (uint32_t*)cost);
}

/* ------------------------------------------------------------------ MIS */

/* Pannotia MIS mega_kernel (pannotia/graph_app/mis/kernel/mis_kernel.cl:220-337;
 * init :78-93): c = -1 undecided, -2 decided; per round mis1 (min priority
 * over undecided neighbours, :245-270), mis2 (strict local minima join the
 * set, s = 2, and mark undecided neighbours in cu, :277-312), stop check,
 * mis3 (commit cu into c, :322-330).  Winners are never adjacent, so the
 * serial sweep gives the parallel result. */
int orc_mis(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
            const float* nv, int32_t* s, uint32_t* rounds) {
  int32_t* c = (int32_t*)malloc(sizeof(int32_t) * (V ? V : 1));
  int32_t* cu = (int32_t*)malloc(sizeof(int32_t) * (V ? V : 1));
  float* mn = (float*)malloc(sizeof(float) * (V ? V : 1));
  if (!c || !cu || !mn) { free(c); free(cu); free(mn); return -2; }
  const uint32_t E = row_ptr[V];
  for (uint32_t i = 0; i < V; ++i) { c[i] = -1; cu[i] = -1; s[i] = 0; }
  uint32_t r = 0;
  for (;;) {
    int stop = 0;
    for (uint32_t t = 0; t < V; ++t) {
      if (c[t] != -1) continue;
      stop = 1;
      uint32_t start = row_ptr[t];
      uint32_t end = (t + 1 < V) ? row_ptr[t + 1] : E; /* :254-257 */
      float m = 99999999.0f;                           /* BIGNUM :68 */
      for (uint32_t e = start; e < end; ++e)
        if (c[col[e]] == -1 && nv[col[e]] < m) m = nv[col[e]];
      mn[t] = m;
    }
    ++r;
    for (uint32_t t = 0; t < V; ++t) {
      if (nv[t] < mn[t] && c[t] == -1) {
        s[t] = 2;
        uint32_t start = row_ptr[t];
        uint32_t end = (t + 1 < V) ? row_ptr[t + 1] : E;
        c[t] = -2;
        for (uint32_t e = start; e < end; ++e)
          if (c[col[e]] == -1) cu[col[e]] = -2;
      }
    }
    if (!stop) break;
    for (uint32_t t = 0; t < V; ++t)
      if (cu[t] == -2) c[t] = cu[t];
  }
  if (rounds) *rounds = r;
  free(c); free(cu); free(mn);
  return 0;
}

/* --------------------------------------------------------------- colour */

/* Pannotia colouring mega_kernel
 * (pannotia/graph_app/color/kernel/color_kernel.cl:159-252): per round every
 * uncoloured vertex takes max priority over uncoloured neighbours -- except
 * that a degree-1 vertex ignores its only neighbour (start != end - 1,
 * :204) -- then uncoloured vertices above that maximum take colour `round`;
 * stop after the round in which no vertex saw an uncoloured neighbour.
 * Colours start at -1 (host, color_gb.cpp:149). */
int orc_color(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
              const float* nv, int32_t* color, uint32_t* rounds) {
  float* mx = (float*)malloc(sizeof(float) * (V ? V : 1));
  if (!mx) return -2;
  const uint32_t E = row_ptr[V];
  for (uint32_t i = 0; i < V; ++i) color[i] = -1;
  int32_t graph_color = 1;
  uint32_t r = 0;
  for (;;) {
    int stop = 0;
    for (uint32_t i = 0; i < V; ++i) {
      if (color[i] != -1) continue;
      uint32_t start = row_ptr[i];
      uint32_t end = (i + 1 < V) ? row_ptr[i + 1] : E;
      float m = -1.0f;
      for (uint32_t e = start; e < end; ++e) {
        if (color[col[e]] == -1 && start != end - 1) {
          stop = 1;
          if (nv[col[e]] > m) m = nv[col[e]];
        }
      }
      mx[i] = m;
    }
    ++r;
    for (uint32_t i = 0; i < V; ++i)
      if (color[i] == -1 && nv[i] > mx[i]) color[i] = graph_color;
    if (!stop) break;
    graph_color++;
  }
  if (rounds) *rounds = r;
  free(mx);
  return 0;
}

/* Closed form of the same colouring, for graphs where the round-by-round
 * restatement is too slow (thousands of rounds on R-MAT): a vertex takes
 * colour 1 + the largest colour among its higher-priority neighbours (0 if
 * none) -- in the kernel it becomes colourable in the first round after all
 * of those are coloured, and no neighbour of lower priority can be coloured
 * before it -- and a degree-1 vertex takes colour 1 (it never looks at its
 * neighbour).  Vertices are visited in decreasing priority (priorities
 * distinct on adjacent vertices, as the kernel needs to terminate). */
static const float* g_prio_sort;
static int cmp_prio_desc(const void* a, const void* b) {
  float x = g_prio_sort[*(const uint32_t*)a], y = g_prio_sort[*(const uint32_t*)b];
  if (x > y) return -1;
  if (x < y) return 1;
  return (*(const uint32_t*)a < *(const uint32_t*)b) ? -1 : 1;
}

int orc_color_fast(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                   const float* nv, int32_t* color, uint32_t* rounds) {
  uint32_t* ord = (uint32_t*)malloc(sizeof(uint32_t) * (V ? V : 1));
  if (!ord) return -2;
  for (uint32_t i = 0; i < V; ++i) { ord[i] = i; color[i] = 0; }
  g_prio_sort = nv;
  qsort(ord, V, sizeof(uint32_t), cmp_prio_desc);
  int32_t mx = 0;
  for (uint32_t k = 0; k < V; ++k) {
    uint32_t v = ord[k];
    int32_t c = 1;
    if (row_ptr[v + 1] - row_ptr[v] != 1) {
      for (uint32_t e = row_ptr[v]; e < row_ptr[v + 1]; ++e) {
        uint32_t u = col[e];
        if (nv[u] > nv[v] && color[u] + 1 > c) c = color[u] + 1;
      }
    }
    color[v] = c;
    if (c > mx) mx = c;
  }
  if (rounds) *rounds = (uint32_t)mx;
  free(ord);
  return 0;
}

/* ------------------------------------------------------------------- BC */

/* Pannotia BC per source, float32, in the order one work-item executes
 * mega_bc_kernel (pannotia/graph_app/bc/kernel/bc_kernel.cl:431-513):
 * clean_1d_array (:452-466), level-synchronous forward sweep with path
 * counts rho (mega_bfs_kernel_func :295-371), backward sweep over the
 * transposed CSR adding rho[w]/rho[i]*(1+sigma[i]) into sigma[w] for
 * predecessors w and sigma[i] into bc[i] for i != s
 * (mega_backtrack_kernel_func :373-428).  No halving for undirected
 * graphs.  bc is accumulated over the given sources (not zeroed here). */
int orc_bc_f32(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
               const uint32_t* trow, const uint32_t* tcol,
               const uint32_t* sources, uint32_t nsrc, float* bc) {
  int32_t* d = (int32_t*)malloc(sizeof(int32_t) * (V ? V : 1));
  float* rho = (float*)malloc(sizeof(float) * (V ? V : 1));
  float* sigma = (float*)malloc(sizeof(float) * (V ? V : 1));
  if (!d || !rho || !sigma) { free(d); free(rho); free(sigma); return -2; }
  const uint32_t E = row_ptr[V];
  for (uint32_t k = 0; k < nsrc; ++k) {
    const uint32_t s = sources[k];
    if (s >= V) { free(d); free(rho); free(sigma); return -1; }
    for (uint32_t i = 0; i < V; ++i) {
      sigma[i] = 0;
      if (i == s) { rho[i] = 1; d[i] = 0; }
      else { rho[i] = 0; d[i] = -1; }
    }
    int32_t ld = 0;
    for (;;) {
      int stop = 0;
      for (uint32_t i = 0; i < V; ++i) {
        if (d[i] != ld) continue;
        uint32_t start = row_ptr[i];
        uint32_t end = (i + 1 < V) ? row_ptr[i + 1] : E;
        for (uint32_t e = start; e < end; ++e) {
          uint32_t w = col[e];
          if (d[w] < 0) { stop = 1; d[w] = ld + 1; }
          if (d[w] == ld + 1) rho[w] = rho[w] + rho[i];
        }
      }
      ld = ld + 1;
      if (!stop) break;
    }
    while (ld > 0) {
      for (uint32_t i = 0; i < V; ++i) {
        if (d[i] != ld - 1) continue;
        uint32_t start = trow[i];
        uint32_t end = (i + 1 < V) ? trow[i + 1] : E;
        for (uint32_t e = start; e < end; ++e) {
          uint32_t w = tcol[e];
          if (d[w] == ld - 2) sigma[w] = sigma[w] + rho[w] / rho[i] * (1 + sigma[i]);
        }
        if (i != s) bc[i] = bc[i] + sigma[i];
      }
      ld = ld - 1;
    }
  }
  free(d); free(rho); free(sigma);
  return 0;
}

/* Independent FP64 Brandes (queue BFS + stack), same definition as the
 * reference (dependencies summed over the given sources, no halving). */
int orc_bc_f64(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
               const uint32_t* sources, uint32_t nsrc, double* bc) {
  int32_t* d = (int32_t*)malloc(sizeof(int32_t) * (V ? V : 1));
  double* sg = (double*)malloc(sizeof(double) * (V ? V : 1));
  double* dl = (double*)malloc(sizeof(double) * (V ? V : 1));
  uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (V ? V : 1));
  if (!d || !sg || !dl || !order) {
    free(d); free(sg); free(dl); free(order);
    return -2;
  }
  for (uint32_t k = 0; k < nsrc; ++k) {
    const uint32_t s = sources[k];
    if (s >= V) { free(d); free(sg); free(dl); free(order); return -1; }
    for (uint32_t i = 0; i < V; ++i) { d[i] = -1; sg[i] = 0; dl[i] = 0; }
    d[s] = 0; sg[s] = 1;
    uint32_t head = 0, tail = 0;
    order[tail++] = s;
    while (head < tail) {
      uint32_t u = order[head++];
      for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
        uint32_t v = col[e];
        if (d[v] < 0) { d[v] = d[u] + 1; order[tail++] = v; }
        if (d[v] == d[u] + 1) sg[v] += sg[u];
      }
    }
    for (uint32_t idx = tail; idx-- > 0;) {
      uint32_t v = order[idx];
      for (uint32_t e = row_ptr[v]; e < row_ptr[v + 1]; ++e) {
        uint32_t u = col[e];
        if (d[u] == d[v] - 1) dl[u] += sg[u] / sg[v] * (1.0 + dl[v]);
      }
      if (v != s) bc[v] += dl[v];
    }
  }
  free(d); free(sg); free(dl); free(order);
  return 0;
}

/* ------------------------------------------------------------------ MST */

static uint32_t uf_find(uint32_t* p, uint32_t x) {
  while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
  return x;
}

/* Minimum spanning forest by Kruskal.  With unique weights the forest is
 * unique, so it equals what the reference's Boruvka computes
 * (lonestar/apps/mst/mst_port.cpp:202-312, mst_common.cl:41-194,
 * mst_port_kernel.cl:35-82): mstwt is a uint32 sum that wraps
 * (mst_port_kernel.cl:69), edges counts unions, components = V - edges.
 * Arcs of weight >= MYINFINITY are never chosen (mst_common.cl:84-88).
 * arc_in_mst (optional) marks the (u < v) arc of every forest edge. */
int orc_mst(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
            const uint32_t* w, uint64_t* weight64, uint32_t* weight32,
            uint32_t* components, uint32_t* edges, uint8_t* arc_in_mst) {
  const uint32_t E = row_ptr[V];
  uint64_t n = 0;
  for (uint32_t u = 0; u < V; ++u)
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e)
      if (u < col[e] && w[e] < ORC_LONESTAR_INF) ++n;
  /* key = weight(32) | arc index(32) */
  uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  uint32_t* src = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
  uint32_t* p = (uint32_t*)malloc(sizeof(uint32_t) * (V ? V : 1));
  if (!key || !src || !p) { free(key); free(src); free(p); return -2; }
  n = 0;
  for (uint32_t u = 0; u < V; ++u)
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
      src[e] = u;
      if (u < col[e] && w[e] < ORC_LONESTAR_INF)
        key[n++] = ((uint64_t)w[e] << 32) | e;
    }
  /* LSD radix sort of the 64-bit keys, 16 bits per pass, skipping passes
   * whose digit is constant */
  {
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    size_t* cnt = (size_t*)malloc(sizeof(size_t) * 65537);
    if (!tmp || !cnt) { free(tmp); free(cnt); free(key); free(src); free(p); return -2; }
    for (int pass = 0; pass < 4; ++pass) {
      const int sh = 16 * pass;
      memset(cnt, 0, sizeof(size_t) * 65537);
      for (uint64_t i = 0; i < n; ++i) cnt[((key[i] >> sh) & 0xFFFF) + 1]++;
      int nonzero = 0;
      for (int d = 1; d <= 65536; ++d) nonzero += cnt[d] != 0;
      if (nonzero <= 1) continue;
      for (int d = 1; d <= 65536; ++d) cnt[d] += cnt[d - 1];
      for (uint64_t i = 0; i < n; ++i) tmp[cnt[(key[i] >> sh) & 0xFFFF]++] = key[i];
      uint64_t* t = key; key = tmp; tmp = t;
    }
    free(tmp);
    free(cnt);
  }
  for (uint32_t i = 0; i < V; ++i) p[i] = i;
  if (arc_in_mst) memset(arc_in_mst, 0, E);
  uint64_t total = 0;
  uint32_t cnt = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint32_t e = (uint32_t)key[i];
    uint32_t a = uf_find(p, src[e]), b = uf_find(p, col[e]);
    if (a == b) continue;
    if (a < b) p[a] = b; else p[b] = a;
    total += w[e];
    ++cnt;
    if (arc_in_mst) arc_in_mst[e] = 1;
  }
  *weight64 = total;
  *weight32 = (uint32_t)total;
  *edges = cnt;
  *components = V - cnt;
  free(key); free(src); free(p);
  return 0;
}

/* dverifysolution (lonestar/apps/sssp/kernel/sssp_common.cl:41-56; BFS
 * variant with unit weights bfs_common.cl:43-60): number of arcs whose
 * relaxation would still improve dist -- 0 for a feasible answer. */
uint64_t orc_verify_dist(uint32_t V, const uint32_t* row_ptr,
                         const uint32_t* col, const uint32_t* w,
                         const uint32_t* dist) {
  uint64_t nerr = 0;
  for (uint32_t u = 0; u < V; ++u)
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
      uint32_t v = col[e];
      uint32_t wt = w ? w[e] : 1;
      if (wt > 0 && dist[u] + wt < dist[v]) ++nerr;
    }
  return nerr;
}

/* Arcs out of reached vertices (the edges/s work unit) and the count of
 * reached vertices. */
uint64_t orc_bfs_reached_arcs(uint32_t V, const uint32_t* row_ptr,
                              const uint32_t* dist, uint32_t inf,
                              uint32_t* reached) {
  uint64_t arcs = 0;
  uint32_t r = 0;
  for (uint32_t u = 0; u < V; ++u)
    if (dist[u] != inf) { ++r; arcs += row_ptr[u + 1] - row_ptr[u]; }
  if (reached) *reached = r;
  return arcs;
}

/* ------------------------------------------------- multi-threaded BFS */

int orc_par_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Level-synchronous BFS, one parallel loop per level (the barrier interval
 * of drelax2, bfs_port_kernel.cl:173-189): the CPU-baseline counterpart of
 * the persistent kernel on all host cores. */
int orc_par_bfs(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                uint32_t src, uint32_t* dist) {
  if (src >= V) return -1;
  uint32_t* cur = (uint32_t*)malloc(sizeof(uint32_t) * (V ? V : 1));
  uint32_t* nxt = (uint32_t*)malloc(sizeof(uint32_t) * (V ? V : 1));
  if (!cur || !nxt) { free(cur); free(nxt); return -2; }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)V; ++i) dist[i] = ORC_LONESTAR_INF;
  dist[src] = 0;
  cur[0] = src;
  uint64_t ncur = 1;
  uint32_t level = 0;
  while (ncur) {
    uint64_t nnext = 0;
    ++level;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)ncur; ++i) {
      uint32_t u = cur[i];
      for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
        uint32_t v = col[e];
        if (__atomic_load_n(&dist[v], __ATOMIC_RELAXED) != ORC_LONESTAR_INF) continue;
        uint32_t expect = ORC_LONESTAR_INF;
        if (__atomic_compare_exchange_n(&dist[v], &expect, level, 0,
                                        __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
          uint64_t slot = __atomic_fetch_add(&nnext, 1, __ATOMIC_RELAXED);
          nxt[slot] = v;
        }
      }
    }
    uint32_t* t = cur; cur = nxt; nxt = t;
    ncur = nnext;
  }
  free(cur); free(nxt);
  return 0;
}
