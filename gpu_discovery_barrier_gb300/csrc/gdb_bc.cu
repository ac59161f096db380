// Betweenness centrality (Brandes) over a list of sources, float32 output.
//
// Semantics of Pannotia mega_bc_kernel (pannotia/graph_app/bc/kernel/bc_kernel.cl:431-513):
// per source s, BFS levels d, shortest-path counts rho (forward,
// mega_bfs_kernel_func :295-371), dependencies sigma with
// sigma[w] += rho[w]/rho[i] * (1 + sigma[i]) for every predecessor w of i
// (backward, mega_backtrack_kernel_func :373-428), and bc[i] += sigma[i]
// for i != s; no halving for undirected graphs.  Path counts are float32
// as in the reference, so they overflow where the reference's do.
//
// GB300 form, one persistent kernel for all sources, one XF barrier per
// level, and each level pair (L, L+1) handled from whichever side has
// fewer arcs -- on power-law graphs one middle level holds most arcs, and
// neither pass walks it:
//  * forward, level L -> L+1, direction-optimising: push -- the level's
//    vertices claim unvisited neighbours (CAS on d) and add their path
//    count into every level-L+1 neighbour's (an FP32 L2 atomic, as the
//    reference's float adds; FP64 ones cost 6 % more of the BC time); pull -- every unvisited vertex sums the path counts of its
//    level-L neighbours and claims itself when the sum is positive.  A
//    pull has no early exit (every parent counts), so it runs only when the
//    unvisited vertices' arcs are fewer than the level's own;
//  * backward, level L (deepest first): levels below the level with the
//    most arcs pull (1 + sigma[w]) / rho[w] from their level-L+1
//    neighbours, levels above it push their own coefficient into their
//    level-L-1 neighbours' FP64 accumulators, and that level itself only
//    finalises: sigma[v] = rho[v] x the sum;
//  * per-arc arithmetic is FP32; pulled sums go through a segmented warp
//    reduction in FP32 whose per-step totals are added in FP64 -- FP64
//    issues at a small fraction of the FP32 rate on this GPU; heavy
//    vertices that pull sum their chunks with FP64 atomics and the last
//    chunk to finish (an acquire-release count-down) writes the vertex;
//  * levels are kept as segments of one light list and one heavy list, so
//    the backward pass visits exactly the reached vertices, and only those
//    are reset between sources;
//  * sigma itself is never stored: each vertex adds it to bc[v] directly.
// The pull forms read in-arcs forward and out-arcs backward; on the
// symmetric graphs this library targets both are the CSR itself.
#include <algorithm>
#include <vector>

#include "gdb_internal.h"
#include "gdb_relaunch.cuh"

namespace {

using namespace gdb;

// Per-vertex state.  st: x = level (int32, -1 = unreached), y = the
// backward coefficient (1 + sigma) / rho (float bits), one 8-byte load for
// the arcs of either pass; rho: the path count, float as the reference's
// (pushes add into it with FP32 L2 atomics); sacc: FP64 accumulator of the
// backward sum of pushed levels.
struct BcWs {
  uint2* st;
  float* rho;
  double* sacc;
  float* bc;
  uint32_t* order;               // light vertices, level segments
  uint4* hc;                     // heavy chunk entries, level segments
  double* hacc;                  // FP64 partial sums per heavy vertex slot
  uint32_t* hleft;               // chunks still to finish per heavy vertex slot
  uint32_t hc_cap;               // chunk entries available
  uint32_t* lev_l;               // light segment start per level
  uint32_t* lev_h;               // heavy chunk-entry start per level
  uint32_t* lev_hc;              // heavy chunks per level
  uint32_t* lev_hv;              // heavy vertex-slot start per level
  unsigned long long* lev_arcs;  // arcs out of each level's vertices
  uint32_t* lcnt;                // [3] light pushes of the next level
  unsigned long long* hcnt;      // [3] (entries << 32) | chunks
  uint32_t* cursor;              // [3]
  uint32_t* hcursor;             // [3]
  const uint32_t* sources;
  uint32_t nsrc;
  uint32_t max_levels;
  int* overflow;
  unsigned long long* stats;     // [0] arcs, [1] supersteps, [2] reached arcs (work units)
};

// Visit one level segment: light groups over order[lb, lb+nl) (begin/edge/
// end hooks) and the level's heavy chunk entries hc[hcb, hcb+nch), whose
// vertex slots start at hvb: heavy(v, slot, chunks_of_v, arc_begin, arc_end).
template <class Begin, class Edge, class End, class Heavy>
__device__ __forceinline__ void visit_level(const GraphView& G, const Warps& W, const BcWs& ws,
                                            uint32_t lb, uint32_t nl, uint32_t hcb, uint32_t hvb,
                                            uint32_t nch, uint32_t* cursor, uint32_t* hcursor,
                                            Begin&& begin, Edge&& edge, End&& end, Heavy&& heavy) {
  const int lane = lane_id();
  const uint32_t k = group_width(nl, W.nwarps);
  WorkTaker lt((nl + k - 1) / k, W, cursor);
  for (uint32_t g = lt.take(); g < lt.n; g = lt.take()) {
    const uint32_t i = g * k + lane;
    const bool act = (uint32_t)lane < k && i < nl;
    const uint32_t v = act ? ld_cg(&ws.order[lb + i]) : 0u;
    begin(v, act);
    __syncwarp();
    group_arcs(G, act, v, edge);
    __syncwarp();
    end(v, act);
  }
  WorkTaker ht(nch, W, hcursor, lt.n);
  for (uint32_t c = ht.take(); c < nch; c = ht.take()) {
    const uint4 ent = ld_cg(&ws.hc[hcb + c]);
    uint32_t b, en;
    chunk_range(G, ent, b, en);
    heavy(ent.x, hvb + ent.z, ent.w, b, en);
  }
}

// visit_level with four 32-arc steps per call of edge4(valid[4], owner[4],
// arc[4]) (group_arcs4): a step's dependent loads are in flight together
// with the next three steps'.
template <class Begin, class Edge4, class End, class Heavy>
__device__ __forceinline__ void visit_level4(const GraphView& G, const Warps& W, const BcWs& ws,
                                             uint32_t lb, uint32_t nl, uint32_t hcb, uint32_t hvb,
                                             uint32_t nch, uint32_t* cursor, uint32_t* hcursor,
                                             Begin&& begin, Edge4&& edge4, End&& end, Heavy&& heavy) {
  const int lane = lane_id();
  const uint32_t k = group_width(nl, W.nwarps);
  WorkTaker lt((nl + k - 1) / k, W, cursor);
  for (uint32_t g = lt.take(); g < lt.n; g = lt.take()) {
    const uint32_t i = g * k + lane;
    const bool act = (uint32_t)lane < k && i < nl;
    const uint32_t v = act ? ld_cg(&ws.order[lb + i]) : 0u;
    begin(v, act);
    __syncwarp();
    group_arcs4(G, act, v, edge4);
    __syncwarp();
    end(v, act);
  }
  WorkTaker ht(nch, W, hcursor, lt.n);
  for (uint32_t c = ht.take(); c < nch; c = ht.take()) {
    const uint4 ent = ld_cg(&ws.hc[hcb + c]);
    uint32_t b, en;
    chunk_range(G, ent, b, en);
    heavy(ent.x, hvb + ent.z, ent.w, b, en);
  }
}

// The four steps of a heavy chunk [b, e) (at most kChunk = 128 arcs).
__device__ __forceinline__ void chunk_steps(uint32_t b, uint32_t e, bool* valid, uint32_t* arc) {
  static_assert(kChunk == 4 * 32, "a chunk is four steps");
  const uint32_t lane = lane_id();
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    arc[j] = b + 32 * j + lane;
    valid[j] = arc[j] < e;
  }
}

__device__ __forceinline__ int32_t level_of(const BcWs& ws, uint32_t v) {
  return (int32_t)__ldcg(reinterpret_cast<const uint32_t*>(&ws.st[v]));
}
__device__ __forceinline__ float rho_of(const BcWs& ws, uint32_t v) {
  return __ldcg(&ws.rho[v]);
}
__device__ __forceinline__ void set_coef(const BcWs& ws, uint32_t v, float c) {
  reinterpret_cast<uint32_t*>(&ws.st[v])[1] = __float_as_uint(c);
}
constexpr uint2 kUnreached = {0xFFFFFFFFu, 0u};
// an empty sum: sums start at -0.0, and -0.0 + x = x for every x >= +0.0
__device__ __forceinline__ bool no_terms(double s) { return s == 0.0 && signbit(s); }

// Heavy-vertex completion: add this chunk's partial sum; the last chunk
// returns true (with the vertex total in *total) and re-arms the counter.
__device__ __forceinline__ bool heavy_done(const BcWs& ws, uint32_t slot, double part,
                                           uint32_t nchunks, double* total) {
  bool last = false;
  if (lane_id() == 0) {
    atomicAdd(&ws.hacc[slot], part);
    // release orders the add before the count-down; the last chunk's
    // acquire makes every chunk's add visible to its read
    last = countdown_acq_rel(&ws.hleft[slot]) == 1u;
    if (last) {
      *total = __ldcg(&ws.hacc[slot]);
      ws.hacc[slot] = -0.0;
      ws.hleft[slot] = nchunks;
    }
  }
  return __shfl_sync(kFull, last, 0);
}

// Loop state of the BC supersteps; every CTA derives the same values.
struct BcState {
  uint32_t si = 0;      // source index
  uint32_t t = 0;       // superstep counter for the rotating slots
  uint32_t L = 0;       // forward level
  uint32_t lbase = 0, hcbase = 0, hvbase = 0;  // level list bases of level L
  uint32_t peak = 0;    // the level with the most arcs
  uint32_t levels = 0;  // non-empty levels of the source
  uint32_t total_l = 0, total_hc = 0;
  unsigned long long vis_arcs = 0, peak_arcs = 0;
};

__device__ __forceinline__ void bc_reset_slot(const BcWs& ws, uint32_t tt, bool leader) {
  if (leader) {
    const int old = (tt + 2) % 3;
    ws.lcnt[old] = 0;
    ws.hcnt[old] = 0;
    ws.cursor[old] = 0;
    ws.hcursor[old] = 0;
  }
}

__device__ __forceinline__ uint32_t bc_degree(const GraphView& G, uint32_t v) {
  return __ldg(&G.row[v + 1]) - __ldg(&G.row[v]);
}

// Before the first source: every vertex unreached, scores 0, counters 0.
__device__ __forceinline__ void bc_init(const GraphView& G, const Warps& W, const BcWs& ws, bool leader) {
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
    ws.st[v] = kUnreached;
    ws.rho[v] = 0.f;
    ws.sacc[v] = -0.0;
    ws.bc[v] = 0.f;
  }
  if (leader) {
    for (int i = 0; i < 3; ++i) {
      ws.lcnt[i] = 0;
      ws.hcnt[i] = 0;
      ws.cursor[i] = 0;
      ws.hcursor[i] = 0;
    }
    *ws.overflow = 0;
    ws.stats[0] = ws.stats[1] = ws.stats[2] = 0;
  }
}

// Seed source src into slot (t+1).
__device__ __forceinline__ void bc_seed(const GraphView& G, const BcWs& ws, uint32_t src, uint32_t t,
                                        bool leader) {
  auto degree = [&](uint32_t v) { return bc_degree(G, v); };
  // -- superstep: seed the source into slot (t+1)
  bc_reset_slot(ws, t, leader);
  if (leader && src >= G.V) {
    // an out-of-range source (only the device-pointer entry points can
    // pass one) seeds nothing: its forward pass finds level 0 empty and it
    // adds nothing, as BFS and SSSP ignore such sources
    ws.lev_arcs[0] = ws.lev_arcs[1] = 0;
    return;
  }
  if (leader) {
    ws.st[src] = make_uint2(0u, 0u);
    ws.rho[src] = 1.f;
    ws.lev_arcs[0] = degree(src);
    ws.lev_arcs[1] = 0;
    const int nx = (t + 1) % 3;
    frontier_seed(G, Frontier{ws.order, ws.hc, &ws.lcnt[nx], &ws.hcnt[nx], G.V, ws.hc_cap,
                              ws.overflow, G.nheavy, ws.hleft, ws.hacc},
                  src);
  }
}

// Forward level S.L (superstep S.t): false when the level is empty (the
// forward pass is over) or the level lists are full; otherwise the level's
// vertices reach level S.L + 1 and S's bases move to that level.
__device__ __forceinline__ bool bc_forward(const GraphView& G, const Warps& W, const BcWs& ws, BcState& S,
                                           double* my, bool leader, unsigned long long& arcs,
                                           unsigned long long& reached_arcs) {
  const int lane = lane_id();
  auto degree = [&](uint32_t v) { return bc_degree(G, v); };
  const uint32_t L = S.L, t = S.t, lbase = S.lbase, hcbase = S.hcbase, hvbase = S.hvbase;
  unsigned long long& vis_arcs = S.vis_arcs;
  unsigned long long& peak_arcs = S.peak_arcs;
  uint32_t& peak = S.peak;
  const int cur = t % 3, nx = (t + 1) % 3;
  const unsigned long long* sc = cta_words<3>([&](unsigned long long* w) {
    w[0] = ld_cg(&ws.lcnt[cur]);
    w[1] = __ldcg(&ws.hcnt[cur]);
    w[2] = __ldcg(&ws.lev_arcs[L]);
  });
  const uint32_t nl = (uint32_t)sc[0];
  const unsigned long long hp = sc[1], mf = sc[2];
  const uint32_t nhv = (uint32_t)(hp >> 32), nch = (uint32_t)hp;
  if (leader && L < ws.max_levels) {
    ws.lev_l[L] = lbase;
    ws.lev_h[L] = hcbase;
    ws.lev_hc[L] = nch;
    ws.lev_hv[L] = hvbase;
  }
  // the slot two supersteps back is free even in the final superstep
  bc_reset_slot(ws, t, leader);
  if (nl == 0 && nhv == 0) return false;
  if (L + 1 >= ws.max_levels) {
    if (leader) *ws.overflow = 1;
    return false;
  }
  // level L+2's arc counter fills during the next superstep
  if (leader) ws.lev_arcs[L + 2] = 0;
  vis_arcs += mf;
  if (mf > peak_arcs) {
    peak_arcs = mf;
    peak = L;
  }
  // direction of L -> L+1, from the same counters in every CTA: a push
  // walks the level's mf arcs, a pull (no early exit: every parent
  // counts) the arcs of every unvisited vertex plus one look at each
  // vertex's level -- the cheaper one runs
  const unsigned long long mu = G.E > vis_arcs ? G.E - vis_arcs : 0ull;
  const bool pull = mu + G.V < mf;
  const uint32_t nlbase = lbase + nl, nhcbase = hcbase + nch, nhvbase = hvbase + nhv;
  Frontier out{ws.order + nlbase, ws.hc + nhcbase, &ws.lcnt[nx], &ws.hcnt[nx], G.V - nlbase,
               ws.hc_cap - nhcbase, ws.overflow, G.nheavy - nhvbase, ws.hleft + nhvbase,
               ws.hacc + nhvbase};
  WarpStage qs = frontier_stage(out, 0);
  const int32_t Li = (int32_t)L;
  unsigned long long next_arcs = 0;  // arcs out of the vertices this lane claims
  if (!pull) {
    // push: one arc of a level-L vertex of path count rv -- claim an
    // unvisited neighbour, add rv to every level-L+1 neighbour
    // four steps of arcs of level-L vertices with path counts rv: claim
    // unvisited neighbours, add rv to every level-L+1 neighbour; the
    // column, level, degree and claim round trips of the four overlap
    auto fwd4 = [&](const bool* valid, const float* rv, const uint32_t* arc) {
      uint32_t u[4], r0[4], r1[4];
      int32_t du[4];
      int old[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        u[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
        arcs += valid[j];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) du[j] = valid[j] ? level_of(ws, u[j]) : -2;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool cl = du[j] == -1;
        // the degree loads go out with the claim, not after it
        r0[j] = cl ? __ldg(&G.row[u[j]]) : 0u;
        r1[j] = cl ? __ldg(&G.row[u[j] + 1]) : 0u;
        old[j] = cl ? atomicCAS(reinterpret_cast<int*>(&ws.st[u[j]]), -1, Li + 1) : -2;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool claimed = du[j] == -1 && old[j] == -1;
        const bool add = du[j] == Li + 1 || claimed || (du[j] == -1 && old[j] == Li + 1);
        if (claimed) next_arcs += r1[j] - r0[j];
        if (add) atomicAdd(&ws.rho[u[j]], rv[j]);
        frontier_push_staged(G, out, qs, claimed, u[j]);
      }
    };
    float rv_lane = 0.f;
    visit_level4(
        G, W, ws, lbase, nl, hcbase, hvbase, nch, &ws.cursor[cur], &ws.hcursor[cur],
        [&](uint32_t v, bool act) {
          rv_lane = act ? rho_of(ws, v) : 0.f;
          if (act) reached_arcs += degree(v);
        },
        [&](const bool* valid, const int* owner, const uint32_t* arc) {
          float rv[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) rv[j] = __shfl_sync(kFull, rv_lane, owner[j]);
          fwd4(valid, rv, arc);
        },
        [&](uint32_t, bool) {},
        [&](uint32_t v, uint32_t, uint32_t, uint32_t b, uint32_t e) {
          const float r = rho_of(ws, v);
          const float rv[4] = {r, r, r, r};
          bool valid[4];
          uint32_t arc[4];
          chunk_steps(b, e, valid, arc);
          fwd4(valid, rv, arc);
          if (lane == 0 && b == __ldg(&G.row[v])) reached_arcs += degree(v);
        });
  } else {
    // pull: every unvisited vertex sums the path counts of its level-L
    // neighbours (all of them) and claims itself when there are any
    for (uint32_t g = W.gwarp; g * 32 < G.V; g += W.nwarps) {
      const uint32_t u = g * 32 + lane;
      const bool unv = u < G.V && level_of(ws, u) == -1;
      my[lane] = 0.0;
      __syncwarp();
      // four steps at once; a neighbour's path count is loaded with its
      // level (and used only when the level is L)
      group_arcs4(G, unv, u, [&](const bool* valid, const int* owner, const uint32_t* arc) {
        uint32_t w[4];
        int32_t lw[4];
        float rw[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          w[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
          arcs += valid[j];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          lw[j] = valid[j] ? level_of(ws, w[j]) : -2;
          rw[j] = valid[j] ? rho_of(ws, w[j]) : 0.f;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) segment_add(my, owner[j], lw[j] == Li ? rw[j] : -0.f);  // -0: no term
      });
      __syncwarp();
      const double sum = my[lane];
      const bool claimed = unv && sum > 0.0;
      if (claimed) {
        ws.st[u].x = (uint32_t)(Li + 1);  // only this lane writes u
        ws.rho[u] = (float)sum;
        next_arcs += degree(u);
      }
      frontier_push_staged(G, out, qs, claimed, u);
    }
    if (leader) reached_arcs += mf;
  }
  qs.flush();
  next_arcs = warp_add_u64(next_arcs);
  if (lane == 0 && next_arcs) atomicAdd(&ws.lev_arcs[L + 1], next_arcs);
  S.lbase = nlbase;
  S.hcbase = nhcbase;
  S.hvbase = nhvbase;
  return true;
}

// Backward level Lb (superstep t) of source src.
__device__ __forceinline__ void bc_backward(const GraphView& G, const Warps& W, const BcWs& ws, int32_t Lb,
                                            uint32_t t, uint32_t peak, uint32_t src, double* my, bool leader,
                                            unsigned long long& arcs) {
  const int lane = lane_id();
  const int cur = t % 3;
  bc_reset_slot(ws, t, leader);
  const unsigned long long* lv = cta_words<5>([&](unsigned long long* w) {
    w[0] = ld_cg(&ws.lev_l[Lb]);
    w[1] = ld_cg(&ws.lev_l[Lb + 1]);
    w[2] = ld_cg(&ws.lev_h[Lb]);
    w[3] = ld_cg(&ws.lev_hv[Lb]);
    w[4] = ld_cg(&ws.lev_hc[Lb]);
  });
  const uint32_t lb = (uint32_t)lv[0], le = (uint32_t)lv[1];
  const uint32_t hcb = (uint32_t)lv[2], hvb = (uint32_t)lv[3];
  const uint32_t nch = (uint32_t)lv[4];
  // sigma of v from the sum of its successors' coefficients.  Sums
  // start at -0.0 and every successor adds at least +0.0, so -0.0 means
  // no successor: sigma stays 0 then even when rho overflowed to inf, as
  // in the reference, which adds nothing; a successor whose own count
  // overflowed (coefficient 0) still gives inf x 0 = NaN, as there
  auto finalize = [&](uint32_t v, float rv, double sum) {
    const float sg = no_terms(sum) ? 0.f : (float)((double)rv * sum);
    set_coef(ws, v, (1.0f + sg) / rv);
    if (v != src) ws.bc[v] += sg;
    return (1.0f + sg) / rv;
  };
  if ((uint32_t)Lb < peak) {
    // pull the coefficients of the level-Lb+1 neighbours
    // four steps at once: the successors' coefficients (-0: no term)
    auto bwd4 = [&](const bool* valid, const uint32_t* arc, float* a) {
      uint32_t c[4];
      uint2 su[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        c[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
        arcs += valid[j];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)  // level and coefficient
        su[j] = valid[j] ? __ldcg(&ws.st[c[j]]) : make_uint2(0xFFFFFFFFu, 0u);
#pragma unroll
      for (int j = 0; j < 4; ++j) a[j] = (int32_t)su[j].x == Lb + 1 ? __uint_as_float(su[j].y) : -0.f;
    };
    float rv_lane = 0.f;
    visit_level4(
        G, W, ws, lb, le - lb, hcb, hvb, nch, &ws.cursor[cur], &ws.hcursor[cur],
        [&](uint32_t v, bool act) {
          my[lane] = -0.0;
          rv_lane = act ? rho_of(ws, v) : 0.f;
        },
        [&](const bool* valid, const int* owner, const uint32_t* arc) {
          float a[4];
          bwd4(valid, arc, a);
#pragma unroll
          for (int j = 0; j < 4; ++j) segment_add(my, owner[j], a[j]);
        },
        [&](uint32_t v, bool act) {
          if (act) finalize(v, rv_lane, my[lane]);
        },
        [&](uint32_t v, uint32_t slot, uint32_t nchunks, uint32_t b, uint32_t e) {
          bool valid[4];
          uint32_t arc[4];
          float a[4];
          chunk_steps(b, e, valid, arc);
          bwd4(valid, arc, a);
          float part = -0.f;
#pragma unroll
          for (int j = 0; j < 4; ++j) part += a[j];
          part = warp_sum_f32(part);
          double tot = 0.0;
          if (heavy_done(ws, slot, part, nchunks, &tot) && lane == 0) finalize(v, rho_of(ws, v), tot);
        });
  } else if ((uint32_t)Lb == peak) {
    // the peak level only finalises: its sums were pushed by level
    // peak + 1 (none when it is the deepest level)
    for (uint32_t k = lb + W.gthread; k < le; k += W.nthreads) {
      const uint32_t v = ws.order[k];
      finalize(v, rho_of(ws, v), __ldcg(&ws.sacc[v]));
    }
    for (uint32_t k = W.gthread; k < nch; k += W.nthreads) {
      const uint4 ent = ld_cg(&ws.hc[hcb + k]);
      if (ent.y == 0) finalize(ent.x, rho_of(ws, ent.x), __ldcg(&ws.sacc[ent.x]));
    }
  } else {
    // finalise from the pushed sum, then push the coefficient into the
    // level-Lb-1 neighbours
    // four steps at once: add the coefficient into level-Lb-1 neighbours
    auto push4 = [&](const bool* valid, const float* cf, const uint32_t* arc) {
      uint32_t u[4];
      int32_t lu[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        u[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
        arcs += valid[j];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) lu[j] = valid[j] ? level_of(ws, u[j]) : -2;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (lu[j] == Lb - 1) atomicAdd(&ws.sacc[u[j]], (double)cf[j]);
    };
    float cf_lane = 0.f;
    visit_level4(
        G, W, ws, lb, le - lb, hcb, hvb, nch, &ws.cursor[cur], &ws.hcursor[cur],
        [&](uint32_t v, bool act) {
          cf_lane = act ? finalize(v, rho_of(ws, v), __ldcg(&ws.sacc[v])) : 0.f;
        },
        [&](const bool* valid, const int* owner, const uint32_t* arc) {
          float cf[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) cf[j] = __shfl_sync(kFull, cf_lane, owner[j]);
          push4(valid, cf, arc);
        },
        [&](uint32_t, bool) {},
        [&](uint32_t v, uint32_t, uint32_t, uint32_t b, uint32_t e) {
          // every chunk derives the same coefficient; the first writes it
          const float rv = rho_of(ws, v);
          const double sum = __ldcg(&ws.sacc[v]);
          float cf;
          if (b == __ldg(&G.row[v])) {
            cf = lane == 0 ? finalize(v, rv, sum) : 0.f;
            cf = __shfl_sync(kFull, cf, 0);
          } else {
            const float sg = no_terms(sum) ? 0.f : (float)((double)rv * sum);
            cf = (1.0f + sg) / rv;
          }
          const float cfs[4] = {cf, cf, cf, cf};
          bool valid[4];
          uint32_t arc[4];
          chunk_steps(b, e, valid, arc);
          push4(valid, cfs, arc);
        });
  }
}

// After a source: reset its reached vertices (superstep t).
__device__ __forceinline__ void bc_reset(const GraphView& G, const Warps& W, const BcWs& ws, uint32_t total_l,
                                         uint32_t total_hc, uint32_t t, bool leader) {
  // -- reset the reached vertices for the next source
  auto reset = [&](uint32_t v) {
    ws.st[v] = kUnreached;
    ws.rho[v] = 0.f;
    ws.sacc[v] = -0.0;
  };
  for (uint32_t k = W.gthread; k < total_l; k += W.nthreads) reset(ws.order[k]);
  for (uint32_t k = W.gthread; k < total_hc; k += W.nthreads) {
    const uint4 ent = ws.hc[k];
    if (ent.y == 0) reset(ent.x);  // one entry per vertex: its first chunk
  }
  bc_reset_slot(ws, t, leader);
}

template <class Sync>
__device__ __forceinline__ void bc_body(Sync& s, const GraphView& G, const BcWs& ws, double* smem) {
  const Warps W = warps_of(s.id(), s.P());
  const bool leader = s.id() == 0 && threadIdx.x == 0;
  double* my = smem + (threadIdx.x & ~31u);
  bc_init(G, W, ws, leader);
  if (!s.sync()) return;
  unsigned long long arcs = 0, reached_arcs = 0;
  BcState S;
  for (S.si = 0; S.si < ws.nsrc; ++S.si) {
    const uint32_t src = ws.sources[S.si];
    bc_seed(G, ws, src, S.t, leader);
    if (!s.sync()) return;
    ++S.t;
    // -- forward levels
    S.L = 0;
    S.lbase = S.hcbase = S.hvbase = 0;
    S.vis_arcs = S.peak_arcs = 0;
    S.peak = 0;
    for (;; ++S.L, ++S.t) {
      if (!bc_forward(G, W, ws, S, my, leader, arcs, reached_arcs)) break;
      if (!s.sync()) return;
    }
    ++S.t;
    S.levels = S.L;  // levels 0 .. L-1 are non-empty
    S.total_l = S.lbase;
    S.total_hc = S.hcbase;
    if (!s.sync()) return;
    // -- backward levels, deepest first.  Pair (L, L+1) is pulled by level
    // L below the peak level and pushed by level L+1 above it.
    for (int32_t Lb = (int32_t)S.levels - 1; Lb >= 0; --Lb, ++S.t) {
      bc_backward(G, W, ws, Lb, S.t, S.peak, src, my, leader, arcs);
      if (!s.sync()) return;
    }
    bc_reset(G, W, ws, S.total_l, S.total_hc, S.t, leader);
    if (!s.sync()) return;
    ++S.t;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    arcs += __shfl_xor_sync(kFull, arcs, o);
    reached_arcs += __shfl_xor_sync(kFull, reached_arcs, o);
  }
  if (lane_id() == 0) {
    if (arcs) atomicAdd(&ws.stats[0], arcs);
    if (reached_arcs) atomicAdd(&ws.stats[2], reached_arcs);
  }
  if (leader) ws.stats[1] = S.t;
}

__global__ void __launch_bounds__(512, 3) k_bc_xf(DiscoveryArgs a, GraphView G, BcWs ws) {
  __shared__ LocalCtx l;
  __shared__ double sacc[1024];
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  bc_body(s, G, ws, sacc);
}

// Relaunch form (bc.cpp:322-420: per source one launch per forward and
// per backward level, the stop flag read back after each): control state
// s[0] = phase (0 seed, 1 forward, 2 backward, 3 reset), s[1..10] = the
// BcState words, s[11] = backward level; d[0..1] = visited and peak arcs.
enum : uint32_t { kBcSeed = 0, kBcForward = 1, kBcBackward = 2, kBcReset = 3 };

__device__ __forceinline__ BcState bc_state_of(const StepCtl& c) {
  BcState S;
  S.si = c.s[1];
  S.t = c.s[2];
  S.L = c.s[3];
  S.lbase = c.s[4];
  S.hcbase = c.s[5];
  S.hvbase = c.s[6];
  S.peak = c.s[7];
  S.levels = c.s[8];
  S.total_l = c.s[9];
  S.total_hc = c.s[10];
  S.vis_arcs = c.d[0];
  S.peak_arcs = c.d[1];
  return S;
}

__device__ __forceinline__ void bc_state_to(const BcState& S, StepCtl& c) {
  c.s[1] = S.si;
  c.s[2] = S.t;
  c.s[3] = S.L;
  c.s[4] = S.lbase;
  c.s[5] = S.hcbase;
  c.s[6] = S.hvbase;
  c.s[7] = S.peak;
  c.s[8] = S.levels;
  c.s[9] = S.total_l;
  c.s[10] = S.total_hc;
  c.d[0] = S.vis_arcs;
  c.d[1] = S.peak_arcs;
}

__global__ void k_bc_rl_init(GraphView G, BcWs ws) {
  bc_init(G, warps_of(blockIdx.x, gridDim.x), ws, blockIdx.x == 0 && threadIdx.x == 0);
}

__global__ void __launch_bounds__(512, 3) k_bc_rl_step(GraphView G, BcWs ws, StepCtl* ctl,
                                                      cudaGraphConditionalHandle cond) {
  __shared__ double sacc[1024];
  const StepCtl& c0 = step_state(ctl);
  const uint32_t phase = c0.s[0];
  const int32_t Lb = (int32_t)c0.s[11];
  BcState S = bc_state_of(c0);
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  double* my = sacc + (threadIdx.x & ~31u);
  const uint32_t src = ws.sources[S.si];
  unsigned long long arcs = 0, reached_arcs = 0;
  bool more_levels = false;
  if (phase == kBcSeed)
    bc_seed(G, ws, src, S.t, leader);
  else if (phase == kBcForward)
    more_levels = bc_forward(G, W, ws, S, my, leader, arcs, reached_arcs);
  else if (phase == kBcBackward)
    bc_backward(G, W, ws, Lb, S.t, S.peak, src, my, leader, arcs);
  else
    bc_reset(G, W, ws, S.total_l, S.total_hc, S.t, leader);
  arcs = warp_add_u64(arcs);
  reached_arcs = warp_add_u64(reached_arcs);
  if (lane_id() == 0) {
    if (arcs) atomicAdd(&ws.stats[0], arcs);
    if (reached_arcs) atomicAdd(&ws.stats[2], reached_arcs);
  }
  // S holds this CTA's view of the next state, the same in every CTA
  step_end(ctl, cond, [&](StepCtl& st) {
    bool more = true;
    ++S.t;
    if (phase == kBcSeed) {
      st.s[0] = kBcForward;
      S.L = 0;
      S.lbase = S.hcbase = S.hvbase = 0;
      S.vis_arcs = S.peak_arcs = 0;
      S.peak = 0;
    } else if (phase == kBcForward) {
      if (more_levels) {
        ++S.L;
      } else {
        S.levels = S.L;  // levels 0 .. L-1 are non-empty
        S.total_l = S.lbase;
        S.total_hc = S.hcbase;
        st.s[0] = S.levels ? kBcBackward : kBcReset;
        st.s[11] = S.levels ? S.levels - 1 : 0;
      }
    } else if (phase == kBcBackward) {
      if (Lb == 0) st.s[0] = kBcReset;
      else st.s[11] = (uint32_t)(Lb - 1);
    } else {
      ++S.si;
      st.s[0] = kBcSeed;
      if (S.si >= ws.nsrc) {
        ws.stats[1] = S.t;
        more = false;
      }
    }
    bc_state_to(S, st);
    return more;
  });
}

// out[v] = the lanes' partial sums, in lane order (deterministic).
struct LaneParts {
  const float* p[gdbi::kMaxLanes];
  int k;
};
__global__ void k_bc_sum(float* out, LaneParts parts, uint32_t V) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < parts.k; ++j) s += parts.p[j][v];
    out[v] = s;
  }
}

}  // namespace

using namespace gdbi;

// Workspace of one BC run (the per-vertex records and accumulators, the
// level lists, heavy-chunk entries and their accumulators, per-level arc
// counts, the counter block).
static size_t bc_layout(const gdb_graph* g, char* base, float* d_bc, const uint32_t* d_sources,
                        uint32_t nsrc, BcWs* ws, char** cnt_out) {
  const uint32_t V = g->V;
  const uint32_t hcap = std::max<uint32_t>(g->nheavy, 1);
  const uint32_t ccap = std::max<uint32_t>(g->nheavy_chunks, 1);
  const uint32_t maxlev = V + 2;
  Bump b;
  const size_t o_st = b.take((size_t)V * 8), o_rho = b.take((size_t)V * 8),
               o_sacc = b.take((size_t)V * 8);
  const size_t o_ord = b.take((size_t)V * 4);
  const size_t o_hc = b.take((size_t)ccap * 16), o_hacc = b.take((size_t)hcap * 8),
               o_hleft = b.take((size_t)hcap * 4);
  const size_t o_ll = b.take((size_t)maxlev * 4), o_lh = b.take((size_t)maxlev * 4),
               o_lhc = b.take((size_t)maxlev * 4), o_lhv = b.take((size_t)maxlev * 4);
  const size_t o_la = b.take((size_t)(maxlev + 2) * 8);
  const size_t o_cnt = b.take(512);
  if (!base) return b.off;
  ws->st = (uint2*)(base + o_st);
  ws->rho = (float*)(base + o_rho);
  ws->sacc = (double*)(base + o_sacc);
  ws->bc = d_bc;
  ws->order = (uint32_t*)(base + o_ord);
  ws->hc = (uint4*)(base + o_hc);
  ws->hc_cap = ccap;
  ws->hacc = (double*)(base + o_hacc);
  ws->hleft = (uint32_t*)(base + o_hleft);
  ws->lev_l = (uint32_t*)(base + o_ll);
  ws->lev_h = (uint32_t*)(base + o_lh);
  ws->lev_hc = (uint32_t*)(base + o_lhc);
  ws->lev_hv = (uint32_t*)(base + o_lhv);
  ws->lev_arcs = (unsigned long long*)(base + o_la);
  char* cnt = base + o_cnt;
  ws->stats = (unsigned long long*)cnt;
  ws->hcnt = (unsigned long long*)(cnt + 64);
  ws->lcnt = (uint32_t*)(cnt + 96);
  ws->cursor = (uint32_t*)(cnt + 112);
  ws->hcursor = (uint32_t*)(cnt + 128);
  ws->overflow = (int*)(cnt + 160);
  ws->sources = d_sources;
  ws->nsrc = nsrc;
  ws->max_levels = maxlev - 1;
  *cnt_out = cnt;
  return b.off;
}

size_t gdbi::bc_workspace_bytes(const gdb_graph* g) {
  return bc_layout(g, nullptr, nullptr, nullptr, 0, nullptr, nullptr);
}

int gdbi::bc_enqueue(gdb_ctx* c, gdb_graph* g, void* wsbase, const uint32_t* d_sources, uint32_t nsrc,
                     float* d_bc, cudaStream_t stream, const gdb::DiscoveryArgs& proto) {
  BcWs ws;
  char* cnt = nullptr;
  bc_layout(g, (char*)wsbase, d_bc, d_sources, nsrc, &ws, &cnt);
  GDB_CUDA(c, cudaMemsetAsync(cnt, 0, 512, stream));
  Shape s;
  int rc = persistent_shape(c, (const void*)k_bc_xf, c->opt.block_size, 0, &s, false);
  if (rc) return rc;
  DiscoveryArgs a = proto;
  a.expected = std::min(s.grid, s.fit);
  k_bc_xf<<<s.grid, c->opt.block_size, 0, stream>>>(a, g->view(), ws);
  GDB_CUDA(c, cudaGetLastError());
  return GDB_OK;
}

// Several sources: contiguous groups of them on concurrent lanes, each
// lane summing into its own array, then one pass adds the lanes' arrays.
// Four lanes: BC's launches are longer and fuller than BFS's and SSSP's
// (R-MAT-22, 16 sources: 16.7 ms on two lanes, 16.2 on four, 18.2 on
// eight, 27.3 on sixteen; on one launch, an earlier build took 20.9 ms).
constexpr uint32_t kBcLanes = 4;

static int bc_lanes(gdb_ctx* c, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc, float* d_bc) {
  const uint32_t k = std::min<uint32_t>(kBcLanes, nsrc);
  const size_t vb = ((size_t)g->V * 4 + 255) & ~size_t(255);
  int occ = 0;
  GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bc_xf, c->opt.block_size, 0));
  std::vector<unsigned long long> st((size_t)k * 4);
  // every lane sums its group into its own array: exactly k lanes
  int rc = run_on_lanes(c, k, (int)k, false, vb + bc_workspace_bytes(g), occ * c->sm_count,
                        [&](gdb_lane& L, uint32_t j) {
                          const uint32_t b = j * nsrc / k, e = (j + 1) * nsrc / k;
                          return bc_enqueue(c, g, L.ws + vb, d_sources + b, e - b, (float*)L.ws,
                                            L.stream, lane_args(c, L));
                        },
                        st.data());
  if (rc) return rc;
  const float ms = (float)c->last.kernel_ms;
  LaneParts parts;
  parts.k = (int)k;
  for (uint32_t j = 0; j < k; ++j) parts.p[j] = (const float*)c->lanes[j].ws;
  GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  k_bc_sum<<<4 * c->sm_count, 256, 0, c->stream>>>(d_bc, parts, g->V);
  GDB_CUDA(c, cudaGetLastError());
  GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  float sum_ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&sum_ms, c->ev0, c->ev1));
  c->last.kernel_ms = ms + sum_ms;
  c->last.launches = k + 1;
  c->last.work_units = 0;
  for (uint32_t j = 0; j < k; ++j) c->last.work_units += st[4 * j + 2];
  return GDB_OK;
}

// Relaunch form: every source on the context stream, one launch per
// superstep.
static int bc_relaunch(gdb_ctx* c, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc, float* d_bc) {
  const size_t wsb = bc_layout(g, nullptr, nullptr, nullptr, 0, nullptr, nullptr);
  const size_t o_ctl = (wsb + 255) & ~size_t(255);
  char* base = (char*)workspace(c, o_ctl + sizeof(StepCtl));
  if (!base) return GDB_ERR_OOM;
  BcWs ws;
  char* cnt = nullptr;
  bc_layout(g, base, d_bc, d_sources, nsrc, &ws, &cnt);
  GDB_CUDA(c, cudaMemsetAsync(cnt, 0, 512, c->stream));
  const int block = c->opt.block_size;
  int grid = 0;
  int rc = step_grid(c, (const void*)k_bc_rl_step, block, &grid);
  if (rc) return rc;
  c->last = gdb_run_stats{};
  StepCtl first{};
  first.s[0] = kBcSeed;
  // per source: a seed, at most V + 1 forward and V backward levels, a reset
  const unsigned long long cap = (unsigned long long)nsrc * (2ull * g->V + 8);
  rc = step_run(c, c->opt.barrier, (const void*)k_bc_rl_init, (const void*)k_bc_rl_step, grid, block,
                (StepCtl*)(base + o_ctl), first, cap, nsrc > 0, g->view(), ws);
  if (rc) return rc;
  unsigned long long* hs = (unsigned long long*)pinned(c, 512);
  if (!hs) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hs, cnt, 512, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (*(int*)((char*)hs + 160)) return set_error(c, GDB_ERR_CAPACITY, "BC list overflow");
  c->last.edges_processed = hs[0];
  c->last.supersteps = (uint32_t)hs[1];
  c->last.work_units = hs[2];
  return GDB_OK;
}

static int bc_run(gdb_ctx* c, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc, float* d_bc) {
  if (!graph_ok(c, g) || !d_bc || (nsrc && !d_sources)) return GDB_ERR_INVALID;
  if (c->opt.barrier == GDB_BARRIER_RELAUNCH || c->opt.barrier == GDB_BARRIER_RELAUNCH_GRAPH)
    return bc_relaunch(c, g, d_sources, nsrc, d_bc);
  if (c->opt.barrier != GDB_BARRIER_XF && c->opt.barrier != GDB_BARRIER_XF_FIXED)
    return set_error(c, GDB_ERR_UNSUPPORTED, "BC runs on the XF barrier or relaunched");
  if (nsrc >= 2) return bc_lanes(c, g, d_sources, nsrc, d_bc);
  char* base = (char*)workspace(c, bc_layout(g, nullptr, nullptr, nullptr, 0, nullptr, nullptr));
  if (!base) return GDB_ERR_OOM;
  BcWs ws;
  char* cnt = nullptr;
  bc_layout(g, base, d_bc, d_sources, nsrc, &ws, &cnt);
  GDB_CUDA(c, cudaMemsetAsync(cnt, 0, 512, c->stream));
  const int block = c->opt.block_size;
  Shape s;
  int rc = persistent_shape(c, (const void*)k_bc_xf, block, 0, &s, c->opt.barrier == GDB_BARRIER_XF);
  if (rc) return rc;
  DiscoveryArgs a = discovery_args(c, s);
  c->last = gdb_run_stats{};
  GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  k_bc_xf<<<s.grid, block, 0, c->stream>>>(a, g->view(), ws);
  GDB_CUDA(c, cudaGetLastError());
  GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  rc = finish_run(c);
  if (rc) return rc;
  unsigned long long* hs = (unsigned long long*)pinned(c, 512);
  if (!hs) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hs, cnt, 512, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (*(int*)((char*)hs + 160)) return set_error(c, GDB_ERR_CAPACITY, "BC list overflow");
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  int n = 0;
  read_participating(c, &n);
  c->last.participating = n;
  c->last.launched = s.grid;
  c->last.launches = 1;
  c->last.kernel_ms = ms;
  c->last.edges_processed = hs[0];
  c->last.supersteps = (uint32_t)hs[1];
  c->last.work_units = hs[2];
  return GDB_OK;
}

extern "C" {

int gdb_bc_device(gdb_ctx* c, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc, float* d_bc) {
  return bc_run(c, g, d_sources, nsrc, d_bc);
}

int gdb_bc(gdb_ctx* c, gdb_graph* g, const uint32_t* sources, uint32_t nsrc, float* bc) {
  if (!graph_ok(c, g) || !bc || (nsrc && !sources)) return GDB_ERR_INVALID;
  for (uint32_t i = 0; i < nsrc; ++i)
    if (sources[i] >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  const size_t nb = (size_t)g->V * 4, sb = std::max<size_t>(nsrc, 1) * 4;
  char* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, nb + sb, c->stream));
  cudaError_t e = nsrc ? cudaMemcpyAsync(d + nb, sources, nsrc * 4, cudaMemcpyHostToDevice, c->stream)
                       : cudaSuccess;
  int rc = e == cudaSuccess ? bc_run(c, g, (const uint32_t*)(d + nb), nsrc, (float*)d)
                            : set_cuda_error(c, e, "sources upload");
  if (rc == GDB_OK) {
    e = cudaMemcpyAsync(bc, d, nb, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "bc read-back");
  }
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

}  // extern "C"
