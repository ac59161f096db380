// Breadth-first search: persistent level-synchronous kernel behind the
// discovery protocol and the XF barrier.
//
// Semantics of LonestarGPU drelax2 (lonestar/apps/bfs/kernel/bfs_port_kernel.cl:146-192,
// processedge2 bfs_common.cl:73-90): dist[src] = 0, a vertex first reached
// in superstep L gets L, unreached vertices keep 1e9.  The reference's
// worklist pushes a vertex once per discovering arc (a benign race,
// bfs_common.cl:85-88) and needs two barriers per level (bfs_port_kernel.cl:177,188);
// here a CAS on dist[v] makes every vertex enter the queue exactly once,
// and three rotating counter sets let one barrier separate levels.
//
// Schedules:
//  * plain: top-down push from a queue every level;
//  * adaptive: direction-optimising -- a level switches to bottom-up pull
//    (every unvisited vertex scans its arcs for a parent at L-1, stopping at
//    the first) when the frontier's arcs exceed the unvisited arcs / 14, and
//    back when the frontier shrinks below V/24.  Levels are identical.
//  * learned: the master CTA evaluates the schedule selector's network
//    inside every barrier (after the last arrival, before the release) on
//    the next level's frontier features and picks push or pull for it;
//  * forced push / pull (trace generation): the same hook records every
//    level's features and duration with the mode fixed.
#include <algorithm>

#include "gdb_internal.h"
#include "gdb_selector.cuh"

namespace {

using namespace gdb;

struct BfsWs {
  uint32_t* dist;
  uint32_t* q[2];
  uint4* hc[2];                // heavy chunk entries
  uint32_t* qcount;            // [3]
  unsigned long long* hcount;  // [3] (heavy vertices << 32) | chunk entries
  uint32_t* cursor;            // [3]
  uint32_t* hcursor;           // [3]
  int* overflow;
  unsigned long long* stats;   // [0] arcs inspected, [1] levels, [2] unvisited arcs, [3] frontier arcs
  uint32_t* mode;              // [3] 0 = top-down, 1 = bottom-up, per level slot
  uint32_t qcap, hcap;
  int adaptive;                // kBfs* schedule below
  uint32_t alpha, beta;        // direction thresholds of the adaptive schedule
  const float* mlp;            // selector parameters (learned schedule)
  gdb_level_trace* trace;      // per-level records (nullable)
  uint32_t trace_cap;
  uint32_t maxdeg;
  const uint32_t* srcs;        // multi-source run when nsrc > 0
  uint32_t nsrc;
  // frontier bitmaps of the pull levels (nullptr: none): two slots of
  // fwords words, slot L & 1 holding bit v iff dist[v] == L while a pull
  // level L reads it; the level stages its first swords words in shared
  // memory
  uint32_t* fbm;
  uint32_t fwords;             // ceil(V / 32) rounded up to a multiple of 4
  uint32_t swords;             // multiple of 4, <= fwords
};

// Frontier bitmap slot of level L (nullptr without bitmaps).
__device__ __forceinline__ uint32_t* fbm_slot(const BfsWs& ws, uint32_t L) {
  return ws.fbm ? ws.fbm + (size_t)(L & 1) * ws.fwords : nullptr;
}

// Level L's bitmap from the level array, one ballot per 32-vertex group
// (every word written, so the slot needs no clearing): run over the grid
// before a pull level that follows a push level.
__device__ __forceinline__ void fbm_build(const GraphView& G, const BfsWs& ws, uint32_t L, const Warps& W) {
  uint32_t* F = fbm_slot(ws, L);
  const uint32_t ngroups = (G.V + 31) / 32;
  for (uint32_t g = W.gwarp; g < ngroups; g += W.nwarps) {
    const uint32_t v = g * 32 + lane_id();
    const unsigned m = __ballot_sync(kFull, v < G.V && ld_cg(&ws.dist[v]) == L);
    if (lane_id() == 0) F[g] = m;
  }
}

// BfsWs::adaptive: plain push, the threshold heuristic, the learned
// selector, and the two fixed modes of trace generation.
enum { kBfsPlain = 0, kBfsHeuristic = 1, kBfsLearned = 2, kBfsForcePush = 3, kBfsForcePull = 4 };

__device__ __forceinline__ unsigned long long ld_cg_u64(const unsigned long long* p) {
  return __ldcg(p);
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// The master CTA's private decision state, in its shared memory: vertices
// and arcs visited so far, the time of the previous decision (traces) and
// the mode in force.
struct DecideState {
  unsigned long long vis_v, vis_a, tprev;
  uint32_t mode;
};

// Decision for level Lnext, taken by the master CTA inside the barrier
// that ends level Lnext - 1 (all of that level's pushes are complete):
// stats[4 + slot] holds the arcs of the frontier in that slot.  Warp 0
// computes; lane 0 writes the mode word ws.mode[0] -- only when the mode
// changes, so that most releases wait for no store of the decision.
__device__ __noinline__ void bfs_decide(const GraphView& G, const BfsWs& ws, const float* smlp,
                                        DecideState* st, uint32_t Lnext, uint32_t nwarps) {
  if (threadIdx.x >= 32) return;
  const int slot = Lnext % 3;
  const uint32_t n = ld_cg(&ws.qcount[slot]);
  const unsigned long long hp = ld_cg_u64(&ws.hcount[slot]);
  const unsigned long long mfi = ld_cg_u64(&ws.stats[4 + slot]);
  const unsigned long long nfi = (unsigned long long)n + (hp >> 32);
  const unsigned long long vis_v = st->vis_v + nfi;
  const unsigned long long vis_a = st->vis_a + mfi;
  const unsigned long long mu = G.E > vis_a ? G.E - vis_a : 0ull;
  const uint32_t prev = st->mode;
  float x[kFeat];
  bfs_features(x, (float)nfi, (float)mfi, (float)mu, (float)G.V, (float)G.E,
               (float)(G.V > vis_v ? G.V - vis_v : 0ull), Lnext, prev, (float)ws.maxdeg, (float)nwarps);
  uint32_t mode = 0;
  if (ws.adaptive == kBfsLearned) {
    // a push level whose frontier holds under 1/1024 of the unvisited arcs
    // stays push without evaluating the network: a pull level would scan
    // every unvisited vertex for a handful of frontier vertices
    if (prev != 0 || mfi * 1024ull >= mu) {
      float out[kOut];
      mlp_warp(smlp, x, out);
      mode = out[kOutPull] < out[kOutPush] ? 1u : 0u;
    }
  } else if (ws.adaptive == kBfsForcePull) {
    mode = 1;
  }
  __syncwarp();
  if (threadIdx.x == 0) {
    if (mode != prev) ws.mode[0] = mode;
    st->mode = mode;
    st->vis_v = vis_v;
    st->vis_a = vis_a;
    if (ws.trace) {
      const unsigned long long now = globaltimer();
      if (Lnext > 0 && Lnext - 1 < ws.trace_cap)
        ws.trace[Lnext - 1].us = (float)(now - st->tprev) * 1e-3f;
      if (Lnext < ws.trace_cap && nfi > 0) {
        for (int i = 0; i < kFeat; ++i) ws.trace[Lnext].x[i] = x[i];
        ws.trace[Lnext].mode = mode;
        ws.trace[Lnext].us = 0.f;
      }
      st->tprev = now;
    }
  }
}

// The queue counts of level slot `cur` (light count, packed heavy count),
// loaded once per CTA into shared memory; every thread of the CTA calls it
// and reads the two words until the next call.
__device__ __forceinline__ const unsigned long long* level_counts(const BfsWs& ws, int cur) {
  __shared__ unsigned long long s[4];
  __syncthreads();
  if (threadIdx.x == 0) {
    s[0] = ld_cg(&ws.qcount[cur]);
    s[1] = ld_cg_u64(&ws.hcount[cur]);
    s[2] = ws.adaptive >= kBfsLearned ? ld_cg(&ws.mode[0]) : 0u;  // the master's decision
    s[3] = ws.adaptive == kBfsHeuristic ? ld_cg_u64(&ws.stats[4 + cur]) : 0ull;  // frontier arcs
  }
  __syncthreads();
  return s;
}

// Top-down expansion of level L into L+1; sc: the level's counts from
// level_counts.  Batched: four 32-arc steps per batch, their column, level
// and claim round trips overlapping -- the selector-hooked kernels (the
// learned schedule of the R-MAT suite: 16-source BFS 2.78 -> 2.64 ms).  The
// plain kernels keep one step per batch: on the 4096^2 grid a vertex has
// four arcs, and there the batch only adds registers that spill
// (50.7 -> 57.5 ms).
template <bool Batched>
__device__ __forceinline__ void bfs_top_down(const GraphView& G, const Warps& W, const BfsWs& ws,
                                             uint32_t L, const unsigned long long* sc,
                                             unsigned long long& arcs, unsigned long long& farcs) {
  const int cur = L % 3, nxt = (L + 1) % 3;
  const uint32_t n = (uint32_t)sc[0];
  const unsigned long long hp = sc[1];
  Frontier out{pick(ws.q, L + 1), pick(ws.hc, L + 1), &ws.qcount[nxt], &ws.hcount[nxt],
               ws.qcap, ws.hcap, ws.overflow};
  WarpStage qs = frontier_stage(out, 0);
  auto edge = [&](bool valid, uint32_t arc) {
    uint32_t u = 0;
    bool want = false;
    if (valid) {
      u = __ldg(&G.col[arc]);
      ++arcs;
      if (ld_cg(&ws.dist[u]) == kInf) {
        // the degree loads are issued before the claim, so that counting
        // the next frontier's arcs adds no round trip after it
        uint32_t r0 = 0, r1 = 0;
        if (ws.adaptive) {
          r0 = __ldg(&G.row[u]);
          r1 = __ldg(&G.row[u + 1]);
        }
        if (atomicCAS(&ws.dist[u], kInf, L + 1) == kInf) {
          want = true;
          farcs += r1 - r0;
        }
      }
    }
    frontier_push_staged(G, out, qs, want, u);
  };
  auto edge4 = [&](const bool* valid, const uint32_t* arc) {
    uint32_t u[4];
    bool want[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      u[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
      arcs += valid[j];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) want[j] = valid[j] && ld_cg(&ws.dist[u[j]]) == kInf;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (want[j]) {
        // the degree loads are issued before the claim, so that counting
        // the next frontier's arcs adds no round trip after it
        uint32_t r0 = 0, r1 = 0;
        if (ws.adaptive) {
          r0 = __ldg(&G.row[u[j]]);
          r1 = __ldg(&G.row[u[j] + 1]);
        }
        want[j] = atomicCAS(&ws.dist[u[j]], kInf, L + 1) == kInf;
        if (want[j]) farcs += r1 - r0;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) frontier_push_staged(G, out, qs, want[j], u[j]);
  };
  if constexpr (Batched) {
    visit_frontier4(G, W, pick(ws.q, L), n, pick(ws.hc, L), hp, &ws.cursor[cur], &ws.hcursor[cur],
                    edge4);
  } else {
    visit_frontier(
        G, W, pick(ws.q, L), n, pick(ws.hc, L), hp, &ws.cursor[cur], &ws.hcursor[cur],
        [&](bool valid, int, uint32_t, uint32_t arc) { edge(valid, arc); },
        [&](bool valid, uint32_t, uint32_t arc) { edge(valid, arc); });
  }
  qs.flush();
}

// Bottom-up step for level L+1: every unvisited vertex looks for a parent
// at level L among its arcs, stopping at the first.  A warp takes 32
// consecutive vertices.  Each lane first probes up to kPullProbe arcs of
// its own vertex, four independent loads at a time; vertices whose lists
// go on are then scanned by the whole warp, 32 arcs per step, one vertex
// after another, leaving at the first step with a hit (so a long list
// costs its length / 32 round trips instead of its length).
//
// With frontier bitmaps a probe tests the neighbour's bit in level L's
// bitmap instead of loading its level.  The bitmap's first swords words
// (the lowest vertex ids: on R-MAT-22 80 % of the vertices' first arcs
// land below id 393,216, a 48 KB prefix, because rows are sorted and
// R-MAT concentrates hubs there) are copied into the CTA's shared memory
// at the level's start with 16-byte loads, so most probes are one
// shared-memory read after the column load instead of a second L2 round
// trip; the rest read the bitmap word from L2.  The level writes level
// L + 1's bitmap whole, one ballot per 32-vertex group, for a following
// pull level; push levels keep no bitmap (fbm_build makes one when a pull
// level follows them).
constexpr uint32_t kPullProbe = 8;

__device__ __forceinline__ void bfs_bottom_up(const GraphView& G, const BfsWs& ws, uint32_t L,
                                              const Warps& W, uint32_t* sbits, unsigned long long& arcs,
                                              unsigned long long& farcs) {
  const int nxt = (L + 1) % 3;
  Frontier out{pick(ws.q, L + 1), pick(ws.hc, L + 1), &ws.qcount[nxt], &ws.hcount[nxt],
               ws.qcap, ws.hcap, ws.overflow};
  WarpStage qs = frontier_stage(out, 0);
  const int lane = lane_id();
  const uint32_t* F = fbm_slot(ws, L);
  uint32_t* Fn = fbm_slot(ws, L + 1);
  const uint32_t sw = F ? ws.swords : 0u;
  if (sw) {
    const uint4* f4 = reinterpret_cast<const uint4*>(F);
    uint4* s4 = reinterpret_cast<uint4*>(sbits);
    for (uint32_t i = threadIdx.x; i < sw / 4; i += blockDim.x) s4[i] = ld_cg(&f4[i]);
    __syncthreads();
  }
  // u in level L's frontier (F written before this level's barrier)
  auto in_frontier = [&](uint32_t u) -> bool {
    if (!F) return ld_cg(&ws.dist[u]) == L;
    const uint32_t wd = u >> 5;
    const uint32_t word = wd < sw ? sbits[wd] : ld_cg(&F[wd]);
    return (word >> (u & 31)) & 1u;
  };
  const uint32_t ngroups = (G.V + 31) / 32;
  for (uint32_t g = W.gwarp; g < ngroups; g += W.nwarps) {
    const uint32_t v = g * 32 + lane;
    bool want = false, open = false;
    uint32_t b = 0, e = 0, deg = 0;
    // an L2 read: another SM's claim in an earlier push level may have
    // changed dist[v] after this SM cached it
    if (v < G.V && ld_cg(&ws.dist[v]) == kInf) {
      b = __ldg(&G.row[v]);
      e = __ldg(&G.row[v + 1]);
      deg = e - b;
      const uint32_t stop = min(e, b + kPullProbe);
      for (uint32_t a = b; a < stop && !want; a += 4) {
        uint32_t u[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) u[k] = a + k < stop ? __ldg(&G.col[a + k]) : kInf;
        if (F) {
          // the four probes' L2 words first (all in flight together), then
          // the staged ones
          uint32_t word[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) word[k] = u[k] != kInf && (u[k] >> 5) >= sw ? ld_cg(&F[u[k] >> 5]) : 0u;
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (u[k] != kInf && (u[k] >> 5) < sw) word[k] = sbits[u[k] >> 5];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (u[k] != kInf) {
              ++arcs;
              if ((word[k] >> (u[k] & 31)) & 1u) want = true;
            }
          }
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (u[k] != kInf) {
              ++arcs;
              if (ld_cg(&ws.dist[u[k]]) == L) want = true;
            }
          }
        }
      }
      b = stop;
      open = !want && stop < e;
    }
    for (unsigned m = __ballot_sync(kFull, open); m; m &= m - 1) {
      const int o = __ffs(m) - 1;
      const uint32_t bb = __shfl_sync(kFull, b, o), ee = __shfl_sync(kFull, e, o);
      bool found = false;
      for (uint32_t a = bb; a < ee; a += 32) {
        bool hit = false;
        if (a + lane < ee) {
          ++arcs;
          hit = in_frontier(__ldg(&G.col[a + lane]));
        }
        if (__any_sync(kFull, hit)) {
          found = true;
          break;
        }
      }
      if (lane == o) want = found;
    }
    if (want) {
      ws.dist[v] = L + 1;  // only this lane writes v
      farcs += deg;
    }
    const unsigned found = __ballot_sync(kFull, want);
    if (Fn && lane == 0) Fn[g] = found;
    frontier_push_staged(G, out, qs, want, v);
  }
  qs.flush();
}

// Hooked: the learned and forced-mode schedules (a decision inside every
// barrier); a separate instantiation keeps the plain kernels' registers.
template <bool Hooked, class Sync>
__device__ __forceinline__ void bfs_body(Sync& s, const GraphView& G, const BfsWs& ws, uint32_t src,
                                         float* smlp, DecideState* dst, uint32_t* sbits) {
  const Warps W = warps_of(s.id(), s.P());
  const bool leader = s.id() == 0 && threadIdx.x == 0;
  constexpr bool hooked = Hooked;
  if constexpr (Hooked) {
    if (ws.adaptive == kBfsLearned)
      for (int i = threadIdx.x; i < kParams; i += blockDim.x) smlp[i] = __ldg(&ws.mlp[i]);
    if (threadIdx.x == 0) *dst = DecideState{0, 0, 0, 0};  // read after the first barrier
  }
  // barrier ending level Lnext - 1; hooked schedules decide level Lnext in it
  auto level_sync = [&](uint32_t Lnext) {
    if constexpr (!Hooked) {
      return s.sync();
    } else {
      return s.sync_hook([&] { bfs_decide(G, ws, smlp, dst, Lnext, W.nwarps); });
    }
  };
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) ws.dist[v] = kInf;
  if (leader) {
    for (int i = 0; i < 3; ++i) {
      ws.qcount[i] = 0;
      ws.hcount[i] = 0;
      ws.cursor[i] = 0;
      ws.hcursor[i] = 0;
      ws.mode[i] = 0;
    }
    *ws.overflow = 0;
    for (int i = 0; i < 8; ++i) ws.stats[i] = 0;
  }
  if (!s.sync()) return;
  const Frontier f0{ws.q[0], ws.hc[0], &ws.qcount[0], &ws.hcount[0], ws.qcap, ws.hcap, ws.overflow};
  if (ws.nsrc) {
    frontier_seed_many(G, f0, W, ws.srcs, ws.nsrc, ws.dist, kInf,
                       hooked ? &ws.stats[4] : (unsigned long long*)nullptr);
  } else if (leader) {
    ws.dist[src] = 0;
    frontier_seed(G, f0, src);
    if (hooked) ws.stats[4] = G.row[src + 1] - G.row[src];
  }
  if (!level_sync(0)) return;
  unsigned long long arcs = 0;
  uint32_t L = 0;
  bool bottom_up = false, prev_bottom_up = false;
  // direction-choice inputs, identical in every CTA: arcs of the frontier
  // (mf) and of the still-unvisited vertices (mu).  acc[k % 3] (stats[4..6])
  // collects the arcs of level k while level k-1 runs.
  unsigned long long mf = ws.nsrc ? 0ull : (unsigned long long)(G.row[src + 1] - G.row[src]);
  unsigned long long mu = G.E - mf;
  for (;; ++L) {
    const int cur = L % 3, old = (L + 2) % 3;
    const unsigned long long* sc = level_counts(ws, cur);
    const uint32_t n = (uint32_t)sc[0];
    const unsigned long long hp = sc[1];
    if (n == 0 && hp == 0) break;
    if (ws.adaptive == kBfsHeuristic) {
      if (L > 0) {
        mf = sc[3];
        mu = mu > mf ? mu - mf : 0;
      }
      const uint32_t nf = n + (uint32_t)(hp >> 32);
      if (!bottom_up && mf > mu / ws.alpha) bottom_up = true;
      else if (bottom_up && nf < G.V / ws.beta) bottom_up = false;
    } else if (hooked) {
      bottom_up = sc[2] != 0;
    }
    if (leader) {
      ws.qcount[old] = 0;
      ws.hcount[old] = 0;
      ws.cursor[old] = 0;
      ws.hcursor[old] = 0;
      ws.stats[4 + old] = 0;
    }
    if (bottom_up && ws.fbm && !prev_bottom_up) {
      // a pull level after a push level (or the first level): its
      // frontier's bitmap from the level array, complete before any probe
      fbm_build(G, ws, L, W);
      if (!s.sync()) return;
    }
    prev_bottom_up = bottom_up;
    unsigned long long farcs = 0;
    if (bottom_up) bfs_bottom_up(G, ws, L, W, sbits, arcs, farcs);
    else bfs_top_down<Hooked>(G, W, ws, L, sc, arcs, farcs);
    if (ws.adaptive) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) farcs += __shfl_xor_sync(kFull, farcs, o);
      if (lane_id() == 0 && farcs) atomicAdd(&ws.stats[4 + (L + 1) % 3], farcs);
    }
    if (!level_sync(L + 1)) return;
  }
  unsigned long long r = arcs;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(kFull, r, o);
  if (lane_id() == 0 && r) atomicAdd(&ws.stats[0], r);
  if (leader) ws.stats[1] = L;
}

// Dynamic shared memory of the traversal kernels: ws.swords words of the
// frontier bitmap staged by pull levels (none when ws.swords is 0).
__global__ void __launch_bounds__(512, 3) k_bfs_xf(DiscoveryArgs a, GraphView G, BfsWs ws, uint32_t src) {
  __shared__ LocalCtx l;
  extern __shared__ uint4 bfs_stage[];
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  bfs_body<false>(s, G, ws, src, nullptr, nullptr, reinterpret_cast<uint32_t*>(bfs_stage));
}

__global__ void __launch_bounds__(512, 3) k_bfs_grid(GraphView G, BfsWs ws, uint32_t src) {
  extern __shared__ uint4 bfs_stage[];
  GridSync s;
  bfs_body<false>(s, G, ws, src, nullptr, nullptr, reinterpret_cast<uint32_t*>(bfs_stage));
}

__global__ void __launch_bounds__(512, 3) k_bfs_xf_sel(DiscoveryArgs a, GraphView G, BfsWs ws,
                                                       uint32_t src) {
  __shared__ LocalCtx l;
  __shared__ float smlp[kParams];
  __shared__ DecideState dst;
  extern __shared__ uint4 bfs_stage[];
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  bfs_body<true>(s, G, ws, src, smlp, &dst, reinterpret_cast<uint32_t*>(bfs_stage));
}

__global__ void __launch_bounds__(512, 3) k_bfs_grid_sel(GraphView G, BfsWs ws, uint32_t src) {
  __shared__ float smlp[kParams];
  __shared__ DecideState dst;
  extern __shared__ uint4 bfs_stage[];
  GridSync s;
  bfs_body<true>(s, G, ws, src, smlp, &dst, reinterpret_cast<uint32_t*>(bfs_stage));
}

// Relaunch mode: init kernel, then one launch per level (no in-kernel barrier).
__global__ void k_bfs_init(GraphView G, BfsWs ws, uint32_t src) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, n = gridDim.x * blockDim.x;
  for (uint32_t v = t; v < G.V; v += n) ws.dist[v] = (v == src) ? 0u : kInf;
  if (t == 0) {
    for (int i = 0; i < 3; ++i) {
      ws.qcount[i] = 0;
      ws.hcount[i] = 0;
      ws.cursor[i] = 0;
      ws.hcursor[i] = 0;
    }
    *ws.overflow = 0;
    ws.stats[0] = ws.stats[1] = 0;
    frontier_seed(G, Frontier{ws.q[0], ws.hc[0], &ws.qcount[0], &ws.hcount[0], ws.qcap, ws.hcap,
                              ws.overflow},
                  src);
  }
}

__global__ void __launch_bounds__(512, 3) k_bfs_level(GraphView G, BfsWs ws, uint32_t L) {
  const int old = (L + 2) % 3;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ws.qcount[old] = 0;
    ws.hcount[old] = 0;
    ws.cursor[old] = 0;
    ws.hcursor[old] = 0;
    ws.stats[1] = L + 1;
  }
  unsigned long long arcs = 0, farcs = 0;
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  bfs_top_down<false>(G, W, ws, L, level_counts(ws, L % 3), arcs, farcs);
  unsigned long long r = arcs;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(kFull, r, o);
  if (lane_id() == 0 && r) atomicAdd(&ws.stats[0], r);
}

// Graph-relaunch mode: the body of a CUDA-graph WHILE node.  The level
// number lives in ctl[0]; the last CTA to finish (ctl[1] counts them)
// advances it and sets the loop condition to "next frontier not empty".
__global__ void __launch_bounds__(512, 3) k_bfs_glevel(GraphView G, BfsWs ws, uint32_t* ctl,
                                                       cudaGraphConditionalHandle cond) {
  __shared__ uint32_t sL;
  if (threadIdx.x == 0) sL = ld_cg(&ctl[0]);
  __syncthreads();
  const uint32_t L = sL;
  const int old = (L + 2) % 3;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ws.qcount[old] = 0;
    ws.hcount[old] = 0;
    ws.cursor[old] = 0;
    ws.hcursor[old] = 0;
  }
  unsigned long long arcs = 0, farcs = 0;
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  bfs_top_down<false>(G, W, ws, L, level_counts(ws, L % 3), arcs, farcs);
  unsigned long long r = arcs;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(kFull, r, o);
  if (lane_id() == 0 && r) atomicAdd(&ws.stats[0], r);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ctl[1], 1u) == gridDim.x - 1) {
      __threadfence();
      const int nxt = (L + 1) % 3;
      const bool more = ld_cg(&ws.qcount[nxt]) != 0 || __ldcg(&ws.hcount[nxt]) != 0;
      ctl[0] = L + 1;
      ctl[1] = 0;
      ws.stats[1] = L + 1;
      cudaGraphSetConditional(cond, more ? 1u : 0u);
    }
  }
}

}  // namespace

using namespace gdbi;

// Words of one frontier bitmap slot of a graph of V vertices.
static uint32_t bitmap_words(uint32_t V) { return ((V + 31) / 32 + 3) & ~3u; }

// Workspace of one BFS run: two light queues, two chunk-entry queues, the
// two frontier bitmap slots, the 512-byte counter block (last: the
// lanes read their statistics at its fixed offset from the end).
static size_t bfs_layout(const gdb_graph* g, char* base, uint32_t* d_dist, BfsWs* ws, char** cnt_out) {
  const uint32_t V = g->V;
  const uint32_t hcap = chunk_capacity(g);
  const uint32_t fwords = bitmap_words(V);
  Bump b;
  const size_t o_q0 = b.take((size_t)V * 4), o_q1 = b.take((size_t)V * 4);
  const size_t o_hc0 = b.take((size_t)hcap * 16), o_hc1 = b.take((size_t)hcap * 16);
  const size_t o_fbm = b.take((size_t)fwords * 8);
  const size_t o_cnt = b.take(512);
  if (!base) return b.off;
  ws->dist = d_dist;
  ws->q[0] = (uint32_t*)(base + o_q0);
  ws->q[1] = (uint32_t*)(base + o_q1);
  ws->hc[0] = (uint4*)(base + o_hc0);
  ws->hc[1] = (uint4*)(base + o_hc1);
  char* cnt = base + o_cnt;
  ws->stats = (unsigned long long*)cnt;                // 8 x u64
  ws->hcount = (unsigned long long*)(cnt + 64);        // 3 x u64
  ws->qcount = (uint32_t*)(cnt + 96);                  // 3
  ws->cursor = (uint32_t*)(cnt + 112);                 // 3
  ws->hcursor = (uint32_t*)(cnt + 128);                // 3
  ws->mode = (uint32_t*)(cnt + 144);                   // 3
  ws->overflow = (int*)(cnt + 160);
  ws->qcap = V;
  ws->hcap = hcap;
  ws->adaptive = kBfsPlain;
  ws->alpha = 14;
  ws->beta = 24;
  ws->mlp = nullptr;
  ws->trace = nullptr;
  ws->trace_cap = 0;
  ws->maxdeg = g->maxdeg;
  ws->srcs = nullptr;
  ws->nsrc = 0;
  ws->fbm = (uint32_t*)(base + o_fbm);
  ws->fwords = fwords;
  ws->swords = 0;
  *cnt_out = cnt;
  return b.off;
}

// The automatic frontier bitmap (pull_bitmap_kb 0): a 16 KB stage
// (131,072 vertex ids) for a traversal that has the GPU to itself; none
// for traversals that share it.  Measured on R-MAT-22, one source per
// call, mean over 16 sources: learned schedule 0.349 -> 0.333 ms with the
// bitmap, threshold schedule 0.324 -> 0.302 ms; 16 sources on four
// concurrent lanes go 2.93 -> 3.02 ms -- their pull levels are
// bandwidth-bound, and the bitmap's build pass costs more than its
// shared-memory probes save.  Stages of 48 KB and more cost occupancy and
// L1 (one source 0.40 / 0.46 ms against 0.36 at 16 KB).
constexpr uint32_t kStageKbAuto = 16;
constexpr uint32_t kStageKbMax = 64;

// Words of the bitmap a pull level stages for schedule `mode` on a graph
// of V vertices (0: no bitmap).
static uint32_t bitmap_stage_words(gdb_ctx* c, int mode, uint32_t V, bool alone) {
  if (mode == kBfsPlain || c->opt.pull_bitmap_kb < 0) return 0;
  const uint32_t kb = c->opt.pull_bitmap_kb ? (uint32_t)c->opt.pull_bitmap_kb : (alone ? kStageKbAuto : 0u);
  return std::min<uint32_t>(kb * 256u, bitmap_words(V));  // both multiples of 4
}

// Frontier bitmaps of ws's schedule (none for plain push, when
// pull_bitmap_kb is -1, or automatically for a traversal sharing the GPU);
// returns the dynamic shared memory, in bytes, the traversal kernel takes.
static void bfs_bitmap(gdb_ctx* c, const gdb_graph* g, BfsWs* ws, bool alone, size_t* smem) {
  ws->swords = bitmap_stage_words(c, ws->adaptive, g->V, alone);
  if (!ws->swords) ws->fbm = nullptr;
  *smem = (size_t)ws->swords * 4;
}

int gdbi::bfs_prepare(gdb_ctx* c) {
  // static + dynamic shared memory above 48 KB needs each kernel's opt-in
  for (const void* k : {(const void*)k_bfs_xf, (const void*)k_bfs_xf_sel, (const void*)k_bfs_grid,
                        (const void*)k_bfs_grid_sel})
    GDB_CUDA(c, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageKbMax * 1024));
  return GDB_OK;
}

int gdbi::traversal_occupancy(gdb_ctx*, int block) {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bfs_xf, block, 0) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return occ;
}

size_t gdbi::bfs_workspace_bytes(const gdb_graph* g) {
  return bfs_layout(g, nullptr, nullptr, nullptr, nullptr);
}

// Graphs whose vertices all have at most this many arcs run the
// direction-optimising schedules as plain push.  A pull level scans every
// unvisited vertex, a push level the frontier's arcs: with d <= 8 arcs per
// vertex a pull can only pay once the unvisited vertices are fewer than
// 8x the frontier, i.e. in the last few levels of a traversal, while the
// per-level cost of the hooked kernel (the next frontier's degree loads,
// the decision inside every barrier, the four-step batches) is paid on
// every level: on the 4096^2 grid (8,191 levels) the learned BFS took
// 91.9 ms against 51.0 ms push-only.
constexpr uint32_t kPushOnlyMaxDeg = 8;

// BfsWs::adaptive for c's schedule on g; the learned one needs a loaded
// selector.
static int bfs_mode(gdb_ctx* c, const gdb_graph* g, int* mode) {
  switch (c->opt.schedule) {
    case GDB_SCHED_ADAPTIVE: *mode = g->maxdeg <= kPushOnlyMaxDeg ? kBfsPlain : kBfsHeuristic; return GDB_OK;
    case GDB_SCHED_LEARNED:
      if (!c->d_mlp) return set_error(c, GDB_ERR_INVALID, "learned schedule without a selector");
      *mode = g->maxdeg <= kPushOnlyMaxDeg ? kBfsPlain : kBfsLearned;
      return GDB_OK;
    default: *mode = kBfsPlain; return GDB_OK;
  }
}

// Enqueue one XF-barrier BFS (counter reset + persistent launch) on
// `stream` without waiting, so that it can be stream-captured.  `proto`
// carries the discovery context and flags the launch synchronises through.
int gdbi::bfs_enqueue(gdb_ctx* c, gdb_graph* g, void* wsbase, const uint32_t* d_srcs, uint32_t nsrc,
                      uint32_t* d_dist, cudaStream_t stream, const gdb::DiscoveryArgs& proto, bool alone) {
  BfsWs ws;
  char* cnt = nullptr;
  bfs_layout(g, (char*)wsbase, d_dist, &ws, &cnt);
  ws.srcs = d_srcs;
  ws.nsrc = nsrc;
  int rc = bfs_mode(c, g, &ws.adaptive);
  if (rc) return rc;
  ws.mlp = c->d_mlp;
  if (c->opt.pull_alpha) ws.alpha = c->opt.pull_alpha;
  if (c->opt.push_beta) ws.beta = c->opt.push_beta;
  GDB_CUDA(c, cudaMemsetAsync(cnt, 0, 512, stream));
  Shape s;
  const bool sel = ws.adaptive >= kBfsLearned;
  auto kx = sel ? k_bfs_xf_sel : k_bfs_xf;
  size_t smem = 0;
  bfs_bitmap(c, g, &ws, alone, &smem);
  rc = persistent_shape(c, (const void*)kx, c->opt.block_size, smem, &s, false);
  if (rc) return rc;
  DiscoveryArgs a = proto;
  a.expected = std::min(s.grid, s.fit);
  kx<<<s.grid, c->opt.block_size, smem, stream>>>(a, g->view(), ws, 0u);
  GDB_CUDA(c, cudaGetLastError());
  return GDB_OK;
}

// force: -1 = c's schedule, else a BfsWs::adaptive value (trace runs).
static int bfs_run(gdb_ctx* c, gdb_graph* g, uint32_t src, const uint32_t* d_srcs, uint32_t nsrc,
                   uint32_t* d_dist, int force = -1, gdb_level_trace* d_trace = nullptr,
                   uint32_t trace_cap = 0) {
  if (!graph_ok(c, g) || !d_dist || (nsrc && !d_srcs)) return GDB_ERR_INVALID;
  if (!nsrc && src >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  BfsWs ws;
  char* cnt = nullptr;
  char* base = (char*)workspace(c, bfs_layout(g, nullptr, nullptr, nullptr, nullptr));
  if (!base) return GDB_ERR_OOM;
  bfs_layout(g, base, d_dist, &ws, &cnt);
  if (force >= 0) {
    ws.adaptive = force;
  } else {
    int rc0 = bfs_mode(c, g, &ws.adaptive);
    if (rc0) return rc0;
  }
  ws.mlp = c->d_mlp;
  ws.trace = d_trace;
  ws.trace_cap = trace_cap;
  if (c->opt.pull_alpha) ws.alpha = c->opt.pull_alpha;
  if (c->opt.push_beta) ws.beta = c->opt.push_beta;
  ws.srcs = d_srcs;
  ws.nsrc = nsrc;
  if (nsrc && c->opt.barrier != GDB_BARRIER_XF && c->opt.barrier != GDB_BARRIER_XF_FIXED &&
      c->opt.barrier != GDB_BARRIER_GRID_SYNC)
    return set_error(c, GDB_ERR_UNSUPPORTED, "multi-source BFS needs a persistent barrier");
  GDB_CUDA(c, cudaMemsetAsync(cnt, 0, 512, c->stream));
  const GraphView G = g->view();
  const int block = c->opt.block_size;
  const int kind = c->opt.barrier;
  c->last = gdb_run_stats{};
  int rc = GDB_OK;
  if (kind == GDB_BARRIER_XF || kind == GDB_BARRIER_XF_FIXED) {
    Shape s;
    auto kx = ws.adaptive >= kBfsLearned ? k_bfs_xf_sel : k_bfs_xf;
    size_t smem = 0;
    bfs_bitmap(c, g, &ws, true, &smem);
    rc = persistent_shape(c, (const void*)kx, block, smem, &s, kind == GDB_BARRIER_XF);
    if (rc) return rc;
    DiscoveryArgs a = discovery_args(c, s);
    GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    kx<<<s.grid, block, smem, c->stream>>>(a, G, ws, src);
    GDB_CUDA(c, cudaGetLastError());
    GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    rc = finish_run(c);
    if (rc) return rc;
    int n = 0;
    read_participating(c, &n);
    c->last.participating = n;
    c->last.launched = s.grid;
    c->last.launches = 1;
  } else if (kind == GDB_BARRIER_GRID_SYNC) {
    int occ = 0;
    auto kg = ws.adaptive >= kBfsLearned ? k_bfs_grid_sel : k_bfs_grid;
    size_t smem = 0;
    bfs_bitmap(c, g, &ws, true, &smem);
    GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kg, block, smem));
    int grid = occ * c->sm_count;
    if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
    GraphView Gc = G;
    BfsWs wsc = ws;
    uint32_t srcc = src;
    void* args[] = {(void*)&Gc, (void*)&wsc, (void*)&srcc};
    GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    GDB_CUDA(c, cudaLaunchCooperativeKernel((const void*)kg, grid, block, args, smem, c->stream));
    GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    GDB_CUDA(c, cudaStreamSynchronize(c->stream));
    c->last.participating = grid;
    c->last.launched = grid;
    c->last.launches = 1;
  } else if (kind == GDB_BARRIER_RELAUNCH) {
    if (ws.adaptive) return set_error(c, GDB_ERR_UNSUPPORTED, "adaptive schedule needs a persistent barrier");
    ws.fbm = nullptr;
    int occ = 0;
    GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bfs_level, block, 0));
    int grid = occ * c->sm_count;
    if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
    uint32_t* h = (uint32_t*)pinned(c, 64);
    if (!h) return GDB_ERR_OOM;
    GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    k_bfs_init<<<grid, block, 0, c->stream>>>(G, ws, src);
    uint32_t launches = 1;
    for (uint32_t L = 0;; ++L) {
      k_bfs_level<<<grid, block, 0, c->stream>>>(G, ws, L);
      ++launches;
      // the stop flag of the reference's relaunch loop: next frontier size
      const int nxt = (L + 1) % 3;
      GDB_CUDA(c, cudaMemcpyAsync(h, &ws.qcount[nxt], 4, cudaMemcpyDeviceToHost, c->stream));
      GDB_CUDA(c, cudaMemcpyAsync(h + 2, &ws.hcount[nxt], 8, cudaMemcpyDeviceToHost, c->stream));
      GDB_CUDA(c, cudaStreamSynchronize(c->stream));
      if (h[0] == 0 && h[2] == 0 && h[3] == 0) break;
    }
    GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    GDB_CUDA(c, cudaStreamSynchronize(c->stream));
    c->last.participating = grid;
    c->last.launched = grid;
    c->last.launches = launches;
  } else if (kind == GDB_BARRIER_RELAUNCH_GRAPH) {
    if (ws.adaptive) return set_error(c, GDB_ERR_UNSUPPORTED, "adaptive schedule needs a persistent barrier");
    ws.fbm = nullptr;
    int occ = 0;
    GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bfs_glevel, block, 0));
    int grid = occ * c->sm_count;
    if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
    uint32_t* ctl = (uint32_t*)(cnt + 192);  // [0] level, [1] CTAs done
    rc = graph_while_run(c, (const void*)k_bfs_init, grid, block, G, ws, src,
                         (const void*)k_bfs_glevel, ctl);
    if (rc) return rc;
    c->last.participating = grid;
    c->last.launched = grid;
  } else {
    return set_error(c, GDB_ERR_UNSUPPORTED, "barrier kind not available for BFS");
  }
  unsigned long long* hs = (unsigned long long*)pinned(c, 512);
  if (!hs) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hs, cnt, 512, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (*(int*)((char*)hs + 160)) return set_error(c, GDB_ERR_CAPACITY, "BFS queue overflow");
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last.kernel_ms = ms;
  c->last.edges_processed = hs[0];
  c->last.supersteps = (uint32_t)hs[1];
  if (kind == GDB_BARRIER_RELAUNCH_GRAPH) c->last.launches = 1 + c->last.supersteps;  // init + levels
  return GDB_OK;
}

extern "C" {

int gdb_bfs_device(gdb_ctx* c, gdb_graph* g, uint32_t src, uint32_t* d_dist) {
  return bfs_run(c, g, src, nullptr, 0, d_dist);
}

int gdb_bfs_multi_device(gdb_ctx* c, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc,
                         uint32_t* d_dist) {
  if (nsrc == 0) return GDB_ERR_INVALID;
  return bfs_run(c, g, 0, d_sources, nsrc, d_dist);
}

int gdb_bfs_multi(gdb_ctx* c, gdb_graph* g, const uint32_t* sources, uint32_t nsrc, uint32_t* dist) {
  if (!graph_ok(c, g) || !dist || !sources || nsrc == 0) return GDB_ERR_INVALID;
  for (uint32_t i = 0; i < nsrc; ++i)
    if (sources[i] >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  const size_t nb = (size_t)g->V * 4;
  char* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, nb + (size_t)nsrc * 4, c->stream));
  cudaError_t e = cudaMemcpyAsync(d + nb, sources, (size_t)nsrc * 4, cudaMemcpyHostToDevice, c->stream);
  int rc = e == cudaSuccess ? bfs_run(c, g, 0, (const uint32_t*)(d + nb), nsrc, (uint32_t*)d)
                            : set_cuda_error(c, e, "sources upload");
  if (rc == GDB_OK) {
    e = cudaMemcpyAsync(dist, d, nb, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "dist read-back");
  }
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

int gdb_bfs_sources_device(gdb_ctx* c, gdb_graph* g, const uint32_t* d_sources, uint32_t n,
                           uint32_t* d_dist) {
  if (!graph_ok(c, g) || !d_sources || !d_dist || n == 0) return GDB_ERR_INVALID;
  const size_t V = g->V;
  if (c->opt.barrier != GDB_BARRIER_XF && c->opt.barrier != GDB_BARRIER_XF_FIXED) {
    // the other barrier kinds: one run after another
    for (uint32_t i = 0; i < n; ++i) {
      const int rc = bfs_run(c, g, 0, d_sources + i, 1, d_dist + i * V);
      if (rc) return rc;
    }
    return GDB_OK;
  }
  int mode = 0;
  int rc = bfs_mode(c, g, &mode);
  if (rc) return rc;
  int occ = 0;
  const void* kx = mode >= kBfsLearned ? (const void*)k_bfs_xf_sel : (const void*)k_bfs_xf;
  const size_t smem = (size_t)bitmap_stage_words(c, mode, g->V, false) * 4;
  GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kx, c->opt.block_size, smem));
  const int fit = occ * c->sm_count;
  return run_on_lanes(c, n, kBfsLanes, true, bfs_workspace_bytes(g), fit, [&](gdb_lane& L, uint32_t i) {
    return bfs_enqueue(c, g, L.ws, d_sources + i, 1, d_dist + i * V, L.stream, lane_args(c, L), false);
  });
}

int gdb_bfs_sources(gdb_ctx* c, gdb_graph* g, const uint32_t* sources, uint32_t n, uint32_t* dist) {
  if (!graph_ok(c, g) || !dist || !sources || n == 0) return GDB_ERR_INVALID;
  for (uint32_t i = 0; i < n; ++i)
    if (sources[i] >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  const size_t nb = (size_t)g->V * 4 * n;
  char* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, nb + (size_t)n * 4, c->stream));
  cudaError_t e = cudaMemcpyAsync(d + nb, sources, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
  int rc = e == cudaSuccess ? gdb_bfs_sources_device(c, g, (const uint32_t*)(d + nb), n, (uint32_t*)d)
                            : set_cuda_error(c, e, "sources upload");
  if (rc == GDB_OK) {
    e = cudaMemcpyAsync(dist, d, nb, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "dist read-back");
  }
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

int gdb_bfs_trace(gdb_ctx* c, gdb_graph* g, uint32_t src, int mode, uint32_t* dist,
                  gdb_level_trace* trace, uint32_t cap, uint32_t* levels) {
  if (!graph_ok(c, g) || mode < 0 || mode > 2 || (cap && !trace)) return GDB_ERR_INVALID;
  if (c->opt.barrier != GDB_BARRIER_XF && c->opt.barrier != GDB_BARRIER_XF_FIXED &&
      c->opt.barrier != GDB_BARRIER_GRID_SYNC)
    return set_error(c, GDB_ERR_UNSUPPORTED, "level traces need a persistent barrier");
  if (mode == 2 && !c->d_mlp) return set_error(c, GDB_ERR_INVALID, "no selector loaded");
  const int force = mode == 0 ? kBfsForcePush : mode == 1 ? kBfsForcePull : kBfsLearned;
  const size_t nb = (size_t)g->V * 4, tb = (size_t)std::max<uint32_t>(cap, 1) * sizeof(gdb_level_trace);
  char* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, nb + tb, c->stream));
  cudaError_t e = cudaMemsetAsync(d + nb, 0, tb, c->stream);
  int rc = e == cudaSuccess ? bfs_run(c, g, src, nullptr, 0, (uint32_t*)d, force,
                                      (gdb_level_trace*)(d + nb), cap)
                            : set_cuda_error(c, e, "trace buffer");
  if (rc == GDB_OK) {
    if (dist) e = cudaMemcpyAsync(dist, d, nb, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && cap) e = cudaMemcpyAsync(trace, d + nb, (size_t)cap * sizeof(gdb_level_trace),
                                                      cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "trace read-back");
    if (levels) *levels = c->last.supersteps;
  }
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

int gdb_bfs(gdb_ctx* c, gdb_graph* g, uint32_t src, uint32_t* dist) {
  if (!graph_ok(c, g) || !dist) return GDB_ERR_INVALID;
  uint32_t* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, (size_t)g->V * 4, c->stream));
  int rc = bfs_run(c, g, src, nullptr, 0, d);
  if (rc == GDB_OK) {
    cudaError_t e = cudaMemcpyAsync(dist, d, (size_t)g->V * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "dist read-back");
  }
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// BFS without any device allocation.
//
// Some callers cannot allocate device memory when they run a traversal: a
// host that has handed all of the GPU's memory to its own pool allocator, a
// plug-in that must not call cudaMalloc/cudaFree because those calls
// synchronise the device behind the host's back, or code on a latency path
// that was budgeted to allocate nothing.  gdb_bfs_noalloc serves them: it
// runs the same persistent BFS kernel as gdb_bfs_device, but its queues,
// counters and discovery/barrier state live in one file-scope device array
// of fixed size, so the call allocates nothing (no context, no graph
// handle, no workspace).  Limits: V <= GDB_NOALLOC_MAX_VERTICES, at most
// kNoAllocMaxCtas participating CTAs; every vertex is walked as a light
// vertex (no heavy-vertex table), which is exact but slower on hubs.
namespace {

constexpr uint32_t kNoAllocMaxV = GDB_NOALLOC_MAX_VERTICES;
constexpr int kNoAllocMaxCtas = 1024;
constexpr int kNoAllocBlock = 512;

// Byte offsets inside the scratch array.
constexpr size_t kNaCtx = 0;                                        // gdb::DeviceCtx
constexpr size_t kNaFlags = 4096;                                   // barrier flag lines
constexpr size_t kNaQ0 = kNaFlags + (size_t)kNoAllocMaxCtas * 128;  // frontier queues
constexpr size_t kNaQ1 = kNaQ0 + (size_t)kNoAllocMaxV * 4;
constexpr size_t kNaBits = kNaQ1 + (size_t)kNoAllocMaxV * 4;        // heavy bitmap (all zero)
constexpr size_t kNaBitsBytes = ((size_t)kNoAllocMaxV / 32 + 64) * 4;
constexpr size_t kNaSmall = kNaBits + kNaBitsBytes;                 // empty heavy tables
constexpr size_t kNaCounters = kNaSmall + 256;                      // BFS counters (512 B)
constexpr size_t kNaTotal = kNaCounters + 512;
static_assert(sizeof(gdb::DeviceCtx) <= kNaFlags, "discovery context does not fit");

// The scratch every GPU that loads this library keeps until the process
// exits (about 8.6 MB).  Host code must not use its name as an address:
// the address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_bfs_noalloc_scratch[kNaTotal];

struct NoAllocDevice {
  bool ready;
  unsigned char* base;  // device address of g_bfs_noalloc_scratch
  int sm_count;
  int occupancy;
  unsigned long long launches;
};
constexpr int kNoAllocMaxDevices = 64;
static NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

// Set-up of the current device: the scratch's address, the launch shape and
// a re-armed discovery context with cleared barrier flags.
static int noalloc_arm(int dev, cudaStream_t stream) {
  NoAllocDevice& d = g_noalloc_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_bfs_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return GDB_ERR_CUDA;
    }
    int sms = 0, occ = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bfs_xf, kNoAllocBlock, 0) != cudaSuccess ||
        occ <= 0) {
      cudaGetLastError();
      return GDB_ERR_CUDA;
    }
    d.base = (unsigned char*)p;
    d.sm_count = sms;
    d.occupancy = occ;
  }
  gdb::DeviceCtx h;
  std::memset(&h, 0, sizeof(h));
  h.poll_open = 1;
  h.stall_after = -1;
  if (cudaMemcpyAsync(d.base + kNaCtx, &h, sizeof(h), cudaMemcpyHostToDevice, stream) != cudaSuccess ||
      cudaMemsetAsync(d.base + kNaFlags, 0, (size_t)kNoAllocMaxCtas * 128, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess) {
    cudaGetLastError();
    return GDB_ERR_CUDA;
  }
  d.ready = true;
  return GDB_OK;
}

}  // namespace

extern "C" int gdb_bfs_noalloc(const uint32_t* d_row_ptr, const uint32_t* d_col, uint32_t V,
                               uint64_t E, uint32_t src, uint32_t* d_dist, void* cuda_stream) {
  if (!d_row_ptr || (E && !d_col) || !d_dist || V == 0 || V > kNoAllocMaxV || src >= V ||
      E >= 0xffffffffull)
    return GDB_ERR_INVALID;
  cudaStream_t stream = (cudaStream_t)cuda_stream;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
    cudaGetLastError();
    return GDB_ERR_CUDA;
  }
  NoAllocDevice& d = g_noalloc_dev[dev];
  if (!d.ready) {
    const int rc = noalloc_arm(dev, stream);
    if (rc) return rc;
  }
  unsigned char* base = d.base;
  // what must start at zero: the counters, the heavy bitmap and tables
  if (cudaMemsetAsync(base + kNaCounters, 0, 512, stream) != cudaSuccess ||
      cudaMemsetAsync(base + kNaSmall, 0, 256, stream) != cudaSuccess ||
      cudaMemsetAsync(base + kNaBits, 0, ((size_t)V / 32 + 2) * 4, stream) != cudaSuccess) {
    cudaGetLastError();
    return GDB_ERR_CUDA;
  }
  GraphView G;
  G.V = V;
  G.E = (uint32_t)E;
  G.row = d_row_ptr;
  G.col = d_col;
  G.w = nullptr;
  G.nheavy = 0;
  G.nheavy_chunks = 0;
  G.heavy_v = (const uint32_t*)(base + kNaSmall);
  G.heavy_chunk = (const uint4*)(base + kNaSmall + 64);
  G.heavy_bits = (const uint32_t*)(base + kNaBits);
  BfsWs ws;
  ws.dist = d_dist;
  ws.q[0] = (uint32_t*)(base + kNaQ0);
  ws.q[1] = (uint32_t*)(base + kNaQ1);
  ws.hc[0] = ws.hc[1] = (uint4*)(base + kNaSmall + 128);
  unsigned char* cnt = base + kNaCounters;
  ws.stats = (unsigned long long*)cnt;
  ws.hcount = (unsigned long long*)(cnt + 64);
  ws.qcount = (uint32_t*)(cnt + 96);
  ws.cursor = (uint32_t*)(cnt + 112);
  ws.hcursor = (uint32_t*)(cnt + 128);
  ws.mode = (uint32_t*)(cnt + 144);
  ws.overflow = (int*)(cnt + 160);
  ws.qcap = V;
  ws.hcap = 1;
  ws.adaptive = 0;
  ws.alpha = 14;
  ws.beta = 24;
  ws.mlp = nullptr;
  ws.trace = nullptr;
  ws.trace_cap = 0;
  ws.maxdeg = 0;
  ws.srcs = nullptr;
  ws.nsrc = 0;
  ws.fbm = nullptr;  // plain push: no frontier bitmaps
  ws.fwords = 0;
  ws.swords = 0;
  DiscoveryArgs a;
  a.ctx = (gdb::DeviceCtx*)(base + kNaCtx);
  a.flags = (int*)(base + kNaFlags);
  a.flag_capacity = kNoAllocMaxCtas;
  a.lock_kind = GDB_LOCK_FREE;
  const int grid = std::min(std::min(d.occupancy * d.sm_count, kNoAllocMaxCtas), 32 * kNoAllocBlock + 1);
  a.expected = grid;
  a.timeout_ns = 2000000000ull;
  a.close_wait_ns = 50000ull;
  a.launch_id = ++d.launches;
  a.xf_release = gdb::kXfPerSlave;
  k_bfs_xf<<<grid, kNoAllocBlock, 0, stream>>>(a, G, ws, src);
  if (cudaGetLastError() != cudaSuccess) return GDB_ERR_CUDA;
  int h[4] = {0, 0, 0, 0};
  int overflow = 0;
  if (cudaMemcpyAsync(h, &a.ctx->status, sizeof(h), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaMemcpyAsync(&overflow, ws.overflow, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess) {
    cudaGetLastError();
    return GDB_ERR_CUDA;
  }
  if (h[0] != 0) {
    // re-arm the discovery context and flags after an error
    noalloc_arm(dev, stream);
    return h[0];
  }
  return overflow ? GDB_ERR_CAPACITY : GDB_OK;
}
