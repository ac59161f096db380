// Single-source shortest paths, two reference entry points.
//
// 1. Worklist SSSP with LonestarGPU semantics (drelax2,
//    lonestar/apps/sssp/kernel/sssp_port_kernel.cl:152-197; processedge2
//    sssp_common.cl:58-81): label-correcting relaxation, atomicMin on the
//    target, push on improvement; arcs of weight >= 1e9 are skipped.  Its
//    fixed point is the exact shortest-distance vector, so the result does
//    not depend on the order of relaxations.  Each superstep pushes a vertex
//    at most once (a stamp array), the queue is the same light/heavy
//    frontier as BFS, and one XF barrier separates supersteps.
//
//    Near-far schedule (delta > 0; Davidson, Baxter, Garland, Owens,
//    "Work-efficient parallel GPU methods for single-source shortest
//    paths", IPDPS 2014): only improvements below the current split enter
//    the next frontier; the others go to a far pile, each vertex at most
//    once per pile.  When the near frontier runs dry, one superstep filters
//    the pile: entries below the old split were settled and are dropped,
//    entries below the new split (pile minimum + delta) form the next near
//    frontier, the rest move to the next pile.  This bounds label-correcting
//    rework to one bucket's width; the fixed point, and so every distance,
//    is the same as the plain schedule's.
//
//    Light/heavy arc split (the edge classification of Meyer and Sanders'
//    delta-stepping, J. Algorithms 49(1), 2003): an arc of weight >= the
//    width cannot end inside the current bucket, so near supersteps relax
//    only the light arcs (weight < width) of their frontier; every vertex a
//    near superstep expands is appended once to a settle list, and when the
//    bucket runs dry one superstep relaxes the heavy arcs of the bucket's
//    vertices, each exactly once, at their final distance.  Re-expansions
//    inside a bucket then touch only light arcs.
//
// 2. Pannotia Jacobi SSSP (mega_kernel, pannotia/graph_app/sssp/kernel/sssp_kernel.cl:170-244):
//    y[v] = min(x[v], min_j data[j] + x[col[j]]) over the CSR given (the
//    reference pulls over the transpose) until nothing changes.  The copy
//    x = y and the separate diff pass of the reference are folded: the two
//    vectors swap roles each iteration and the sweep itself raises the
//    change flag, so an iteration costs one barrier instead of three.
#include <algorithm>

#include "gdb_internal.h"
#include "gdb_relaunch.cuh"
#include "gdb_selector.cuh"

namespace {

using namespace gdb;

struct SsspWs {
  uint32_t* dist;
  uint32_t* stamp;             // superstep + 1 in which the vertex was pushed
  // persistent kernels: distance and push stamp of a vertex in one word,
  // (distance << 32) | stamp, so one 64-bit atomicMin both improves the
  // distance and tells whether the vertex is already queued; the result is
  // copied into dist at the end
  unsigned long long* key;
  uint32_t* q[2];
  uint4* hc[2];                // heavy chunk entries
  uint32_t* qcount;            // [3]
  unsigned long long* hcount;  // [3]
  uint32_t* cursor;            // [3]
  uint32_t* hcursor;           // [3]
  int* overflow;
  unsigned long long* stats;   // [0] arcs, [1] supersteps
  uint32_t qcap, hcap;
  const uint32_t* srcs;        // multi-source run when nsrc > 0
  uint32_t nsrc;
  // near-far schedule (delta > 0): far piles ping-pong by phase parity,
  // their counters and minima rotate over three slots by phase % 3
  uint32_t delta;
  uint32_t* far[2];
  uint32_t* farcount;          // [3]
  uint32_t* farmin;            // [3]
  uint32_t* farmark;           // phase + 1 of the pile holding the vertex
  // light/heavy split (light < kInf): near supersteps relax arcs of weight
  // < light; expanded vertices go once to the settle list (stamp = phase +
  // 1 marks them), a run-long append-only frontier whose entries of one
  // bucket are relaxed over their heavy arcs when the bucket runs dry
  uint32_t light;
  uint32_t* sq;
  uint4* shc;
  uint32_t* sqcount;
  unsigned long long* shcount;
  unsigned long long* sarcs;   // heavy arcs of the settle list's vertices
  // direction of the settle supersteps (split only): kSettleRule -- the
  // side with fewer heavy arcs; kSettleLearned -- the selector, evaluated
  // at the start of each settle superstep; forced push / pull (settle
  // traces)
  int settle;
  const float* mlp;
  gdb_level_trace* trace;      // one record per settle superstep (nullable)
  uint32_t trace_cap;
  uint32_t maxdeg;
};

enum { kSettleRule = 0, kSettleLearned = 1, kSettlePush = 2, kSettlePull = 3 };

// CTA 0's settle trace bookkeeping, in its shared memory.
struct SettleState {
  unsigned long long t0;  // start of the settle superstep of the open record
  uint32_t k;             // settle supersteps recorded so far
  uint32_t open;          // a record waits for its duration
};

__device__ __forceinline__ unsigned long long sssp_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Direction of a settle superstep (1 = pull), chosen at its start by warp
// 0 of every CTA from the counters every CTA has just read after the
// barrier -- identical inputs and operations, so every CTA reaches the same
// decision and no barrier waits for it: the network's cheaper output of
// push / pull on the settle's features (decision kind 3), or the forced
// mode of a trace run.  CTA 0 opens the trace record.
__device__ __noinline__ uint32_t settle_choose(const GraphView& GH, const SsspWs& ws, SettleState* st, uint32_t phase, uint32_t sn, uint32_t hn,
                                               unsigned long long an, uint32_t sdone, uint32_t hdone,
                                               unsigned long long adone, uint32_t nwarps, bool master) {
  const unsigned long long mf = an - adone;
  const unsigned long long mu = GH.E > an ? GH.E - an : 0ull;
  const float nf = (float)(sn - sdone) + (float)(hn - hdone);
  float x[kFeat];
  bfs_features(x, nf, (float)mf, (float)mu, (float)GH.V, (float)GH.E,
               (float)(GH.V > sn ? GH.V - sn : 0u), phase, 3u, (float)ws.maxdeg, (float)nwarps);
  uint32_t mode = ws.settle == kSettlePull ? 1u : 0u;
  if (ws.settle == kSettleLearned) {
    // where one side holds over 16x the other's work (the push's heavy
    // arcs against the pull's open heavy arcs plus one look at every
    // vertex) the choice is plain and the network, a few microseconds on
    // the superstep's critical path, is not asked (on R-MAT-22 it agrees
    // with this on every such settle; evaluated on all ten it made the
    // 16-source SSSP 0.8 ms slower)
    const double push_work = (double)mf, pull_work = (double)mu + GH.V;
    if (push_work > 16.0 * pull_work) {
      mode = 1;
    } else if (pull_work > 16.0 * push_work) {
      mode = 0;
    } else {
      // parameters straight from global memory: asked a few times per run,
      // they would cost the kernel 6.8 KB of shared memory per CTA, and the
      // smaller L1 that leaves made the whole SSSP 2-4 % slower
      float out[kOut];
      mlp_warp(ws.mlp, x, out);
      mode = out[kOutPull] < out[kOutPush] ? 1u : 0u;
    }
  }
  if (master && threadIdx.x == 0 && ws.trace && st->k < ws.trace_cap) {
    for (int i = 0; i < kFeat; ++i) ws.trace[st->k].x[i] = x[i];
    ws.trace[st->k].mode = mode;
    ws.trace[st->k].us = 0.f;
    st->t0 = sssp_clock();
    st->open = 1;
  }
  return mode;
}

// Warp-aggregated append of the lanes' `want` vertices to the far pile of
// `phase` (each vertex at most once per pile, so V entries suffice).
__device__ __forceinline__ void far_push(const SsspWs& ws, uint32_t phase, bool want, uint32_t v) {
  const unsigned m = __ballot_sync(kFull, want);
  if (!m) return;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane_id() == leader) base = atomicAdd(&ws.farcount[phase % 3], (uint32_t)__popc(m));
  base = __shfl_sync(kFull, base, leader);
  if (want) {
    const uint32_t slot = base + __popc(m & lanemask_lt());
    if (slot < ws.qcap) pick(ws.far, phase)[slot] = v;
    else atomicExch(ws.overflow, 1);
  }
}

template <bool Keyed>
__device__ __forceinline__ uint32_t dist_of(const SsspWs& ws, uint32_t v) {
  if constexpr (Keyed) {
    return (uint32_t)(ld_cg(&ws.key[v]) >> 32);
  } else {
    return ld_cg(&ws.dist[v]);
  }
}

// The counts of superstep slot `cur` and of the far pile of `phase`
// (light, packed heavy, pile size, pile minimum), loaded once per CTA into
// shared memory; every thread of the CTA calls it and reads the words
// until the next call.
__device__ __forceinline__ const unsigned long long* step_counts(const SsspWs& ws, int cur,
                                                                 uint32_t phase) {
  __shared__ unsigned long long s[7];
  __syncthreads();
  if (threadIdx.x == 0) {
    s[0] = ld_cg(&ws.qcount[cur]);
    s[1] = __ldcg(&ws.hcount[cur]);
    s[2] = ws.delta ? ld_cg(&ws.farcount[phase % 3]) : 0u;
    s[3] = ws.delta ? ld_cg(&ws.farmin[phase % 3]) : 0u;
    const bool split = ws.light < kInf;
    s[4] = split ? ld_cg(ws.sqcount) : 0u;
    s[5] = split ? (uint32_t)__ldcg(ws.shcount) : 0u;
    s[6] = split ? __ldcg(ws.sarcs) : 0ull;
  }
  __syncthreads();
  return s;
}

// One relaxation superstep over frontier (q[0, n), chunk entries hc[0,
// nch)): arcs of weight in [wlo, whi) are relaxed; improvements below
// `split` are pushed to the next frontier (slot L + 1), the others to the
// far pile of `phase`.  With `record`, every expanded vertex not yet in the
// settle list of this phase is appended to it (its work entries laid out
// for graph GR, the view the settle superstep walks).
template <bool Keyed>
__device__ __forceinline__ void sssp_sweep(const GraphView& G, const GraphView& GR, const Warps& W,
                                           const SsspWs& ws, uint32_t L, uint32_t split,
                                           uint32_t phase,
                                           const uint32_t* q, uint32_t n, const uint4* hc,
                                           uint32_t nch, uint32_t wlo, uint32_t whi, bool record,
                                           unsigned long long& arcs) {
  const int cur = L % 3, nxt = (L + 1) % 3;
  Frontier out{pick(ws.q, L + 1), pick(ws.hc, L + 1), &ws.qcount[nxt], &ws.hcount[nxt],
               ws.qcap, ws.hcap, ws.overflow};
  const uint32_t pile = phase + 1;
  const int lane = lane_id();
  // queue appends (next frontier, far pile, settle list) are staged per
  // warp in shared memory; the pile minimum is a per-lane register folded
  // in once at the end
  WarpStage qs = frontier_stage(out, 0);
  WarpStage fs{warp_stage(1), pick(ws.far, phase), &ws.farcount[phase % 3], ws.qcap, ws.overflow};
  uint32_t fmin = 0xFFFFFFFFu;   // lane's smallest far improvement
  auto relax = [&](bool valid, uint32_t du, uint32_t arc) {
    uint32_t v = 0, nd = 0;
    bool want = false, far = false;
    if (valid) {
      v = __ldg(&G.col[arc]);
      const uint32_t wt = __ldg(&G.w[arc]);
      if (wt >= wlo && wt < whi) {
        ++arcs;
        nd = du + wt;
        if constexpr (Keyed) {
          // the stamp part: L + 1 for a near push, 0 for a far one (so a
          // later near improvement in the same superstep still pushes); at
          // an equal distance the older, smaller stamp stays
          if (nd < dist_of<true>(ws, v)) {
            const unsigned long long k =
                ((unsigned long long)nd << 32) | (nd < split ? (unsigned long long)(L + 1) : 0ull);
            const unsigned long long old = atomicMin(&ws.key[v], k);
            if (nd < (uint32_t)(old >> 32)) {
              if (nd < split) want = (uint32_t)old != L + 1;
              else far = true;  // the pile minimum must see every far improvement
            }
          }
        } else if (nd < ld_cg(&ws.dist[v])) {
          const uint32_t old = atomicMin(&ws.dist[v], nd);
          if (nd < old) {
            if (nd < split) {
              want = ld_cg(&ws.stamp[v]) != L + 1 && atomicExch(&ws.stamp[v], L + 1) != L + 1;
            } else {
              // the pile minimum must see every far improvement, queued or not
              far = true;
            }
          }
        }
      }
    }
    frontier_push_staged(G, out, qs, want, v);
    if (ws.delta && __any_sync(kFull, far)) {
      // improvements of vertices already in the pile lower its minimum too
      if (far) fmin = min(fmin, nd);
      const bool add = far && ld_cg(&ws.farmark[v]) != pile && atomicExch(&ws.farmark[v], pile) != pile;
      fs.add(add, v);
    }
  };
  // four 32-arc steps at once (Keyed): column/weight loads, key loads and
  // atomicMins of the four steps in flight together
  auto relax4 = [&](const bool* valid, const uint32_t* du4, const uint32_t* arc) {
    uint32_t v[4], nd[4];
    bool in[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = valid[k] ? __ldg(&G.col[arc[k]]) : 0u;
      const uint32_t wt = valid[k] ? __ldg(&G.w[arc[k]]) : kInf;
      in[k] = valid[k] && wt >= wlo && wt < whi;
      nd[k] = du4[k] + wt;
      arcs += in[k];
    }
    uint32_t cur[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) cur[k] = in[k] ? dist_of<true>(ws, v[k]) : 0u;
    unsigned long long old[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const bool t = in[k] && nd[k] < cur[k];
      old[k] = t ? atomicMin(&ws.key[v[k]], ((unsigned long long)nd[k] << 32) |
                                                 (nd[k] < split ? (unsigned long long)(L + 1) : 0ull))
                 : 0ull;
      in[k] = t;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      bool want = false, far = false;
      if (in[k] && nd[k] < (uint32_t)(old[k] >> 32)) {
        if (nd[k] < split) want = (uint32_t)old[k] != L + 1;
        else far = true;
      }
      frontier_push_staged(G, out, qs, want, v[k]);
      if (ws.delta && __any_sync(kFull, far)) {
        if (far) fmin = min(fmin, nd[k]);
        const bool add = far && ld_cg(&ws.farmark[v[k]]) != pile && atomicExch(&ws.farmark[v[k]], pile) != pile;
        fs.add(add, v[k]);
      }
    }
  };
  const Frontier settle{ws.sq, ws.shc, ws.sqcount, ws.shcount, ws.qcap, ws.hcap, ws.overflow};
  WarpStage ss = frontier_stage(settle, 2);
  // a vertex is in a superstep's frontier at most once, so a plain mark
  // store dedupes expansions across the bucket's supersteps
  unsigned long long rec_arcs = 0;  // heavy arcs of the vertices this lane records
  auto remember = [&](bool act, uint32_t u) {
    const bool add = act && ld_cg(&ws.stamp[u]) != pile;
    if (add) {
      ws.stamp[u] = pile;
      rec_arcs += __ldg(&GR.row[u + 1]) - __ldg(&GR.row[u]);
    }
    frontier_push_staged(GR, settle, ss, add, u);
  };
  // light groups: each lane reads its own vertex's distance once
  const uint32_t k = group_width(n, W.nwarps);
  WorkTaker lt((n + k - 1) / k, W, &ws.cursor[cur]);
  for (uint32_t g = lt.take(); g < lt.n; g = lt.take()) {
    const uint32_t i = g * k + lane;
    const bool act = (uint32_t)lane < k && i < n;
    const uint32_t u = act ? ld_cg(&q[i]) : 0u;
    const uint32_t du = act ? dist_of<Keyed>(ws, u) : 0u;
    if (record) remember(act, u);
    if constexpr (Keyed) {
      group_arcs4(G, act, u, [&](const bool* valid, const int* owner, const uint32_t* arc) {
        uint32_t d4[4];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) d4[kk] = __shfl_sync(kFull, du, owner[kk]);
        relax4(valid, d4, arc);
      });
    } else {
      group_arcs(G, act, u, [&](bool valid, int owner, uint32_t arc) {
        relax(valid, __shfl_sync(kFull, du, owner), arc);
      });
    }
  }
  WorkTaker ht(nch, W, &ws.hcursor[cur], lt.n);
  for (uint32_t c = ht.take(); c < nch; c = ht.take()) {
    const uint4 ent = ld_cg(&hc[c]);
    const uint32_t du = dist_of<Keyed>(ws, ent.x);
    if (record) remember(lane == 0 && ent.y == 0, ent.x);
    uint32_t b, en;
    chunk_range(G, ent, b, en);
    if constexpr (Keyed) {
      bool valid[4];
      uint32_t arc[4], d4[4];
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        arc[kk] = b + 32 * kk + lane;
        valid[kk] = arc[kk] < en;
        d4[kk] = du;
      }
      relax4(valid, d4, arc);
    } else {
      range_arcs(b, en, [&](bool valid, uint32_t arc) { relax(valid, du, arc); });
    }
  }
  qs.flush();
  if (record) {
    ss.flush();
    rec_arcs = warp_add_u64(rec_arcs);
    if (lane == 0 && rec_arcs) atomicAdd(ws.sarcs, rec_arcs);
  }
  if (ws.delta) {
    fs.flush();
    fmin = __reduce_min_sync(kFull, fmin);
    if (lane == 0 && fmin != 0xFFFFFFFFu) atomicMin(&ws.farmin[phase % 3], fmin);
  }
}

// Settle by pull, the other direction of a settle superstep: every vertex
// at or beyond the split takes the minimum of dist(v) + w over its heavy
// in-arcs v -> u (GT: the heavy half transposed) from vertices below the
// split (all final).  It replaces walking the
// heavy arcs of the bucket's vertices when the unsettled vertices hold
// fewer heavy arcs -- on power-law graphs the first bucket holds the hubs
// and most arcs.  Same fixed point: each relaxation it applies is one the
// push would apply, and arcs from earlier buckets can no longer improve.
__device__ __forceinline__ void settle_pull(const GraphView& GT, const Warps& W, const SsspWs& ws,
                                            uint32_t split, uint32_t phase, uint32_t* smin,
                                            unsigned long long& arcs) {
  const int lane = lane_id();
  const uint32_t pile = phase + 1;
  WarpStage fs{warp_stage(1), pick(ws.far, phase), &ws.farcount[phase % 3], ws.qcap, ws.overflow};
  uint32_t fmin = 0xFFFFFFFFu;
  uint32_t* my = smin + (threadIdx.x & ~31u);
  for (uint32_t g = W.gwarp; g * 32 < GT.V; g += W.nwarps) {
    const uint32_t u = g * 32 + lane;
    const uint32_t du = u < GT.V ? dist_of<true>(ws, u) : 0u;
    const bool open = u < GT.V && du >= split;
    my[lane] = 0xFFFFFFFFu;
    __syncwarp();
    // four steps at once: their column, weight and distance loads overlap
    group_arcs4(GT, open, u, [&](const bool* valid, const int* owner, const uint32_t* arc) {
      uint32_t v[4], w[4], dv[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        v[j] = valid[j] ? __ldg(&GT.col[arc[j]]) : 0u;
        w[j] = valid[j] ? __ldg(&GT.w[arc[j]]) : 0u;
        arcs += valid[j];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) dv[j] = valid[j] ? dist_of<true>(ws, v[j]) : 0xFFFFFFFFu;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (dv[j] < split) atomicMin(&my[owner[j]], dv[j] + w[j]);
    });
    __syncwarp();
    const uint32_t nd = my[lane];
    const bool better = open && nd < du;
    if (better) {
      ws.key[u] = (unsigned long long)nd << 32;  // a far improvement; only this lane writes u
      fmin = min(fmin, nd);
    }
    const bool add = better && ld_cg(&ws.farmark[u]) != pile;
    if (add) ws.farmark[u] = pile;
    fs.add(add, u);
  }
  fs.flush();
  fmin = __reduce_min_sync(kFull, fmin);
  if (lane == 0 && fmin != 0xFFFFFFFFu) atomicMin(&ws.farmin[phase % 3], fmin);
}

// Phase change of the near-far schedule: split the far pile of `phase`
// into the next near frontier ([lo, split)), dropped settled entries
// (< lo) and the pile of phase + 1 (>= split).
__device__ __forceinline__ void far_filter(const GraphView& G, const Warps& W, const SsspWs& ws,
                                           uint32_t L, uint32_t phase, uint32_t lo, uint32_t split,
                                           uint32_t fn) {
  const int nxt = (L + 1) % 3;
  Frontier out{pick(ws.q, L + 1), pick(ws.hc, L + 1), &ws.qcount[nxt], &ws.hcount[nxt],
               ws.qcap, ws.hcap, ws.overflow};
  const uint32_t* pile = pick(ws.far, phase);
  const int lane = lane_id();
  uint32_t fmin = 0xFFFFFFFFu;  // lane's smallest kept distance
  for (uint32_t base = W.gwarp * 32; base < fn; base += W.nwarps * 32) {
    const uint32_t i = base + lane;
    const bool act = i < fn;
    const uint32_t v = act ? ld_cg(&pile[i]) : 0u;
    const uint32_t d = act ? dist_of<true>(ws, v) : 0u;
    const bool near = act && d >= lo && d < split;
    const bool keep = act && d >= split;
    if (keep) ws.farmark[v] = phase + 2;
    frontier_push(G, out, near, v);
    far_push(ws, phase + 1, keep, v);
    if (keep) fmin = min(fmin, d);
  }
  fmin = __reduce_min_sync(kFull, fmin);
  if (lane == 0 && fmin != 0xFFFFFFFFu) atomicMin(&ws.farmin[(phase + 1) % 3], fmin);
}

// G: the arcs near supersteps relax (all arcs, or the light half under
// the split); GH: the heavy half the settle supersteps relax, GT the same
// transposed (split only).
// Hooked: the settle direction comes from settle_choose (learned and trace
// schedules); a separate instantiation keeps the plain kernels' registers.
template <bool Hooked, class Sync>
__device__ __forceinline__ void sssp_body(Sync& s, const GraphView& G, const GraphView& GH,
                                          const GraphView& GT, const SsspWs& ws, uint32_t src,
                                          uint32_t* smin, SettleState* sst) {
  const Warps W = warps_of(s.id(), s.P());
  const bool leader = s.id() == 0 && threadIdx.x == 0;
  const bool split_arcs = ws.light < kInf;
  if constexpr (Hooked) {
    if (threadIdx.x == 0) *sst = SettleState{0, 0, 0};  // read after the first barrier
  }
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
    ws.key[v] = (unsigned long long)kInf << 32;
    if (ws.delta) ws.farmark[v] = 0;
    if (split_arcs) ws.stamp[v] = 0;
  }
  if (leader) {
    for (int i = 0; i < 3; ++i) {
      ws.qcount[i] = 0;
      ws.hcount[i] = 0;
      ws.cursor[i] = 0;
      ws.hcursor[i] = 0;
      if (ws.delta) {
        ws.farcount[i] = 0;
        ws.farmin[i] = 0xFFFFFFFFu;
      }
    }
    *ws.overflow = 0;
    *ws.sqcount = 0;
    *ws.shcount = 0;
    *ws.sarcs = 0;
    ws.stats[0] = ws.stats[1] = ws.stats[2] = 0;
  }
  if (!s.sync()) return;
  const Frontier f0{ws.q[0], ws.hc[0], &ws.qcount[0], &ws.hcount[0], ws.qcap, ws.hcap, ws.overflow};
  if (ws.nsrc) {
    // one push per distinct in-range source (a CAS claims it)
    const int lane = lane_id();
    for (uint32_t base = W.gwarp * 32; base < ws.nsrc; base += W.nwarps * 32) {
      const uint32_t i = base + lane;
      bool want = i < ws.nsrc;
      const uint32_t v = want ? __ldg(&ws.srcs[i]) : 0u;
      if (v >= G.V) want = false;
      if (want) want = atomicCAS(&ws.key[v], (unsigned long long)kInf << 32, 0ull) ==
                       (unsigned long long)kInf << 32;
      frontier_push(G, f0, want, v);
    }
  } else if (leader) {
    ws.key[src] = 0;
    frontier_seed(G, f0, src);
  }
  if (!s.sync()) return;
  unsigned long long arcs = 0;
  uint32_t L = 0;
  // every CTA derives split and phase from the same counters after each
  // barrier, so they stay uniform across the grid
  uint32_t split = ws.delta ? ws.delta : 0xFFFFFFFFu, phase = 0;
  // settle-list entries (light vertices, chunk entries) already relaxed,
  // and the heavy arcs of all vertices recorded by then
  uint32_t sdone = 0, hdone = 0;
  unsigned long long adone = 0;
  const uint32_t whi = split_arcs ? ws.light : kInf;
  for (;; ++L) {
    const int cur = L % 3, old = (L + 2) % 3;
    const unsigned long long* sc = step_counts(ws, cur, phase);
    if constexpr (Hooked) {
      // a settle superstep ended at the barrier just passed: its duration
      if (s.id() == 0 && threadIdx.x == 0 && sst->open) {
        if (sst->k < ws.trace_cap) ws.trace[sst->k].us = (float)(sssp_clock() - sst->t0) * 1e-3f;
        sst->open = 0;
        ++sst->k;
      }
    }
    const bool dry = sc[0] == 0 && sc[1] == 0;
    const uint32_t sn = (uint32_t)sc[4], hn = (uint32_t)sc[5];
    const bool unsettled = sn > sdone || hn > hdone;
    if (dry && !unsettled && (!ws.delta || sc[2] == 0)) break;
    if (leader) {
      ws.qcount[old] = 0;
      ws.hcount[old] = 0;
      ws.cursor[old] = 0;
      ws.hcursor[old] = 0;
    }
    if (dry && unsettled) {
      // the bucket is settled: relax the heavy arcs of its vertices once,
      // from whichever side holds fewer of them (the pull also looks at
      // every vertex's distance once)
      const unsigned long long an = sc[6];
      const unsigned long long open_arcs = GH.E > an ? GH.E - an : 0ull;
      bool pull = open_arcs + GH.V < an - adone;
      if constexpr (Hooked) {
        __shared__ uint32_t sdir;
        if (threadIdx.x < 32) {
          const uint32_t d = settle_choose(GH, ws, sst, phase, sn, hn, an, sdone, hdone, adone, W.nwarps,
                                           s.id() == 0);
          if (threadIdx.x == 0) sdir = d;
        }
        __syncthreads();
        pull = sdir != 0;
      }
      if (pull) {
        settle_pull(GT, W, ws, split, phase, smin, arcs);
      } else {
        sssp_sweep<true>(GH, GH, W, ws, L, split, phase, ws.sq + sdone, sn - sdone, ws.shc + hdone,
                         hn - hdone, ws.light, kInf, false, arcs);
      }
      sdone = sn;
      hdone = hn;
      adone = an;
    } else if (dry) {
      const uint32_t lo = split;
      const unsigned long long nx = (unsigned long long)max(lo, (uint32_t)sc[3]) + ws.delta;
      split = (uint32_t)min(nx, 0xFFFFFFFFull);
      if (leader) {
        // slot (phase + 2) % 3 was last read by the previous phase change
        ws.farcount[(phase + 2) % 3] = 0;
        ws.farmin[(phase + 2) % 3] = 0xFFFFFFFFu;
      }
      far_filter(G, W, ws, L, phase, lo, split, (uint32_t)sc[2]);
      ++phase;
    } else {
      sssp_sweep<true>(G, GH, W, ws, L, split, phase, pick(ws.q, L), (uint32_t)sc[0],
                       pick(ws.hc, L), (uint32_t)sc[1], 0u, whi, split_arcs, arcs);
    }
    if (!s.sync()) return;
  }
  // the distances, out of the keys (every key is final after the last barrier)
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads)
    ws.dist[v] = (uint32_t)(ld_cg(&ws.key[v]) >> 32);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) arcs += __shfl_xor_sync(kFull, arcs, o);
  if (lane_id() == 0 && arcs) atomicAdd(&ws.stats[0], arcs);
  if (leader) {
    ws.stats[1] = L;
    ws.stats[2] = phase;
  }
}

// Two CTAs per SM at up to 64 registers: the four-step batches and the
// bucket state keep more values live than 40 registers hold (R-MAT-22 at
// the automatic width: 2.20 ms per source at three CTAs per SM, 1.97 ms).
__global__ void __launch_bounds__(512, 2) k_sssp_xf(DiscoveryArgs a, GraphView G, GraphView GH,
                                                     GraphView GT, SsspWs ws, uint32_t src) {
  __shared__ LocalCtx l;
  __shared__ uint32_t smin[512];
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  sssp_body<false>(s, G, GH, GT, ws, src, smin, nullptr);
}

__global__ void __launch_bounds__(512, 2) k_sssp_xf_sel(DiscoveryArgs a, GraphView G, GraphView GH,
                                                         GraphView GT, SsspWs ws, uint32_t src) {
  __shared__ LocalCtx l;
  __shared__ uint32_t smin[512];
  __shared__ SettleState sst;
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  sssp_body<true>(s, G, GH, GT, ws, src, smin, &sst);
}

__global__ void __launch_bounds__(512, 2) k_sssp_grid(GraphView G, GraphView GH, GraphView GT,
                                                       SsspWs ws, uint32_t src) {
  __shared__ uint32_t smin[512];
  GridSync s;
  sssp_body<false>(s, G, GH, GT, ws, src, smin, nullptr);
}

// Relaunch modes: an init launch, then one launch per superstep; the last
// CTA of a superstep advances ctl[0] and publishes whether another
// superstep follows -- as the loop condition of a CUDA-graph WHILE node
// (ctl[2] == 0) or as the stop word ctl[3] that the host loop reads back
// (ctl[2] == 1).
__global__ void k_sssp_init(GraphView G, SsspWs ws, uint32_t src) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, n = gridDim.x * blockDim.x;
  for (uint32_t v = t; v < G.V; v += n) {
    ws.dist[v] = v == src ? 0u : kInf;
    ws.stamp[v] = 0;
  }
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

__global__ void __launch_bounds__(512, 3) k_sssp_glevel(GraphView G, SsspWs ws, uint32_t* ctl,
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
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  unsigned long long arcs = 0;
  const unsigned long long* sc = step_counts(ws, L % 3, 0);
  sssp_sweep<false>(G, G, W, ws, L, 0xFFFFFFFFu, 0, pick(ws.q, L), (uint32_t)sc[0], pick(ws.hc, L),
                    (uint32_t)sc[1], 0u, kInf, false, arcs);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) arcs += __shfl_xor_sync(kFull, arcs, o);
  if (lane_id() == 0 && arcs) atomicAdd(&ws.stats[0], arcs);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ctl[1], 1u) == gridDim.x - 1) {
      __threadfence();
      const int nxt = (L + 1) % 3;
      const bool more = ld_cg(&ws.qcount[nxt]) != 0 || __ldcg(&ws.hcount[nxt]) != 0;
      ctl[0] = L + 1;
      ctl[1] = 0;
      ctl[3] = more ? 0u : 1u;
      ws.stats[1] = L + 1;
      if (ctl[2] == 0) cudaGraphSetConditional(cond, more ? 1u : 0u);
    }
  }
}

// ------------------------------------------------------------- Jacobi

struct JacobiWs {
  int32_t* x[2];
  uint32_t* cursor;    // [3]
  uint32_t* hcursor;   // [3]
  uint32_t* changed;   // [3]
  unsigned long long* stats;  // [0] arcs, [1] iterations
};

// One Jacobi iteration reading x[k&1] and writing x[(k+1)&1].  Light
// vertices: per-owner minimum in a shared-memory slot; heavy vertices:
// chunk minima combined with atomicMin -- valid without re-initialising the
// target because costs only decrease (its stale content is an older,
// larger cost of the same vertex).  Arithmetic is the reference's int32
// (data[j] + x[col[j]], sssp_kernel.cl:219-220).
__device__ __forceinline__ bool jacobi_iter(const GraphView& G, const JacobiWs& ws, uint32_t k,
                                            int* smin, unsigned long long& arcs) {
  const int cur = k % 3;
  const int32_t* xo = pick(ws.x, k);
  int32_t* xn = pick(ws.x, k + 1);
  const int lane = lane_id();
  int* my = smin + (threadIdx.x & ~31u);
  bool changed = false;
  int32_t xv = 0;
  sweep_light(
      G, &ws.cursor[cur],
      [&](uint32_t v, bool in_range) {
        xv = in_range ? ld_cg(&xo[v]) : 0;
        my[lane] = xv;
        return true;
      },
      [&](bool valid, int owner, uint32_t arc) {
        if (valid) {
          ++arcs;
          const int32_t c = (int32_t)__ldg(&G.w[arc]) + ld_cg(&xo[__ldg(&G.col[arc])]);
          if (c < my[owner]) atomicMin(&my[owner], c);
        }
      },
      [&](uint32_t v, bool act) {
        if (act) {
          const int32_t m = my[lane];
          xn[v] = m;
          if (m != xv) changed = true;
        }
      });
  sweep_heavy(G, &ws.hcursor[cur], [&](uint32_t v, uint32_t, uint32_t, uint32_t b, uint32_t e) {
    const int32_t xov = ld_cg(&xo[v]);
    int32_t m = xov;
    for (uint32_t a0 = b; a0 < e; a0 += 32) {
      const uint32_t a = a0 + lane;
      if (a < e) {
        ++arcs;
        const int32_t c = (int32_t)__ldg(&G.w[a]) + ld_cg(&xo[__ldg(&G.col[a])]);
        m = min(m, c);
      }
    }
    m = __reduce_min_sync(kFull, m);
    if (lane == 0) {
      atomicMin(&xn[v], m);
      if (m < xov) changed = true;
    }
  });
  return changed;
}

template <class Sync>
__device__ __forceinline__ void jacobi_body(Sync& s, const GraphView& G, const JacobiWs& ws,
                                            uint32_t src, int* smin) {
  const Warps W = warps_of(s.id(), s.P());
  const bool leader = s.id() == 0 && threadIdx.x == 0;
  // vector_init (sssp_kernel.cl:111-132) into both buffers
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
    const int32_t init = v == src ? 0 : GDB_PANNOTIA_BIG;
    ws.x[0][v] = init;
    ws.x[1][v] = init;
  }
  if (leader) {
    for (int i = 0; i < 3; ++i) ws.cursor[i] = ws.hcursor[i] = ws.changed[i] = 0;
    ws.stats[0] = ws.stats[1] = 0;
  }
  if (!s.sync()) return;
  unsigned long long arcs = 0;
  uint32_t k = 0;
  // the reference iterates k = 1 .. num_rows-1 (sssp_kernel.cl:185)
  for (; k + 1 < G.V; ++k) {
    // changed[k % 3] is written in iteration k and read after its barrier,
    // so the slot cleared now is the one of iteration k - 2
    const int cur = k % 3, old = (k + 1) % 3;
    if (leader) ws.cursor[old] = ws.hcursor[old] = ws.changed[old] = 0;
    const bool ch = jacobi_iter(G, ws, k, smin, arcs);
    cta_or(ch, &ws.changed[cur], 1u);
    if (!s.sync()) return;
    if (cta_words<1>([&](unsigned long long* w) { w[0] = ld_cg(&ws.changed[cur]); })[0] == 0) {
      ++k;
      break;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) arcs += __shfl_xor_sync(kFull, arcs, o);
  if (lane_id() == 0 && arcs) atomicAdd(&ws.stats[0], arcs);
  // k iterations ran; the answer is the vector the last one read,
  // x[(k - 1) & 1] -- the reference's host reads x (sssp_gb.cpp:310), which
  // lags y by one iteration when the num_rows - 1 cap ends the loop
  if (leader) ws.stats[1] = k;
}

__global__ void __launch_bounds__(512, 3) k_jacobi_xf(DiscoveryArgs a, GraphView G, JacobiWs ws, uint32_t src) {
  __shared__ LocalCtx l;
  __shared__ int smin[1024];
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  jacobi_body(s, G, ws, src, smin);
}

// Relaunch form (sssp.cpp:290-344: one launch per iteration, the stop flag
// read back after it): vector_init, then one jacobi_iter per launch; the
// control block holds the iteration number k.
__global__ void k_jacobi_rl_init(GraphView G, JacobiWs ws, uint32_t src) {
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
    const int32_t init = v == src ? 0 : GDB_PANNOTIA_BIG;
    ws.x[0][v] = init;
    ws.x[1][v] = init;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int i = 0; i < 3; ++i) ws.cursor[i] = ws.hcursor[i] = ws.changed[i] = 0;
    ws.stats[0] = ws.stats[1] = 0;
  }
}

__global__ void __launch_bounds__(512, 3) k_jacobi_rl_step(GraphView G, JacobiWs ws, uint32_t src,
                                                          StepCtl* ctl, cudaGraphConditionalHandle cond) {
  __shared__ int smin[1024];
  const uint32_t k = step_state(ctl).s[0];
  const int cur = k % 3, old = (k + 1) % 3;
  if (blockIdx.x == 0 && threadIdx.x == 0) ws.cursor[old] = ws.hcursor[old] = ws.changed[old] = 0;
  unsigned long long arcs = 0;
  const bool ch = jacobi_iter(G, ws, k, smin, arcs);
  cta_or(ch, &ws.changed[cur], 1u);
  arcs = warp_add_u64(arcs);
  if (lane_id() == 0 && arcs) atomicAdd(&ws.stats[0], arcs);
  step_end(ctl, cond, [&](StepCtl& st) {
    const uint32_t k1 = st.s[0] + 1;  // iterations run
    st.s[0] = k1;
    ws.stats[1] = k1;
    // the reference's loop: k = 1 .. num_rows-1 while something changed
    return __ldcg(&ws.changed[cur]) != 0 && k1 + 1 < G.V;
  });
}

// Sum, count and maximum of the usable weights (< kInf), for the automatic
// bucket width of the near-far schedule and its light/heavy split.
// Sum, count and maximum of the usable weights (< kInf): a stream with no
// gather behind it, read as 16-byte groups, four groups in flight per
// thread (a 4-byte grid-stride loop keeps one load per thread in flight
// and reached a tenth of HBM bandwidth: 0.37 ms for R-MAT-22's 513 MB).
// The weights not on a 16-byte boundary at either end are read singly.
__global__ void k_weight_sum(const uint32_t* w, unsigned long long E, unsigned long long* out) {
  unsigned long long sum = 0, cnt = 0;
  uint32_t mx = 0;
  auto take = [&](uint32_t x) {
    if (x < kInf) {
      sum += x;
      ++cnt;
      mx = max(mx, x);
    }
  };
  const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  const unsigned long long nthreads = (unsigned long long)gridDim.x * blockDim.x;
  // w is 4-byte aligned: 0-3 weights before the first 16-byte boundary
  const unsigned long long head = std::min<unsigned long long>(E, ((16u - ((uintptr_t)w & 15u)) & 15u) / 4u);
  const unsigned long long n4 = (E - head) / 4;
  const uint4* w4 = reinterpret_cast<const uint4*>(w + head);
  if (tid < head) take(__ldg(&w[tid]));
  for (unsigned long long i = tid; i < n4; i += 4 * nthreads) {
    uint4 q[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const unsigned long long j = i + k * nthreads;
      q[k] = j < n4 ? __ldg(&w4[j]) : make_uint4(kInf, kInf, kInf, kInf);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      take(q[k].x);
      take(q[k].y);
      take(q[k].z);
      take(q[k].w);
    }
  }
  const unsigned long long t0 = head + 4 * n4;  // 0-3 weights after the last whole group
  if (t0 + tid < E) take(__ldg(&w[t0 + tid]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_xor_sync(kFull, sum, o);
    cnt += __shfl_xor_sync(kFull, cnt, o);
    mx = max(mx, __shfl_xor_sync(kFull, mx, o));
  }
  if (lane_id() == 0 && cnt) {
    atomicAdd(&out[0], sum);
    atomicAdd(&out[1], cnt);
    atomicMax(&out[2], (unsigned long long)mx);
  }
}

}  // namespace

using namespace gdbi;

// Workspace of one worklist SSSP run: stamps, two light queues, two
// chunk-entry queues, far piles and marks, the distance keys, the settle
// list (light queue + chunk entries), the 512-byte counter block.
static size_t sssp_layout(const gdb_graph* g, char* base, uint32_t* d_dist, SsspWs* ws, char** cnt_out) {
  const uint32_t V = g->V;
  const uint32_t hcap = chunk_capacity(g);
  Bump b;
  const size_t o_st = b.take((size_t)V * 4);
  const size_t o_q0 = b.take((size_t)V * 4), o_q1 = b.take((size_t)V * 4);
  const size_t o_hc0 = b.take((size_t)hcap * 16), o_hc1 = b.take((size_t)hcap * 16);
  const size_t o_f0 = b.take((size_t)V * 4), o_f1 = b.take((size_t)V * 4), o_fm = b.take((size_t)V * 4);
  const size_t o_key = b.take((size_t)V * 8);
  const size_t o_sq = b.take((size_t)V * 4), o_shc = b.take((size_t)hcap * 16);
  const size_t o_cnt = b.take(512);
  if (!base) return b.off;
  ws->dist = d_dist;
  ws->stamp = (uint32_t*)(base + o_st);
  ws->key = (unsigned long long*)(base + o_key);
  ws->far[0] = (uint32_t*)(base + o_f0);
  ws->far[1] = (uint32_t*)(base + o_f1);
  ws->farmark = (uint32_t*)(base + o_fm);
  ws->q[0] = (uint32_t*)(base + o_q0);
  ws->q[1] = (uint32_t*)(base + o_q1);
  ws->hc[0] = (uint4*)(base + o_hc0);
  ws->hc[1] = (uint4*)(base + o_hc1);
  char* cnt = base + o_cnt;
  ws->stats = (unsigned long long*)cnt;
  ws->hcount = (unsigned long long*)(cnt + 64);
  ws->qcount = (uint32_t*)(cnt + 96);
  ws->cursor = (uint32_t*)(cnt + 112);
  ws->hcursor = (uint32_t*)(cnt + 128);
  ws->overflow = (int*)(cnt + 160);
  // cnt + 192: graph-relaunch control words
  ws->farcount = (uint32_t*)(cnt + 224);               // 3
  ws->farmin = (uint32_t*)(cnt + 240);                 // 3
  ws->sqcount = (uint32_t*)(cnt + 256);
  ws->shcount = (unsigned long long*)(cnt + 264);
  ws->sarcs = (unsigned long long*)(cnt + 272);
  ws->sq = (uint32_t*)(base + o_sq);
  ws->shc = (uint4*)(base + o_shc);
  ws->settle = kSettleRule;
  ws->mlp = nullptr;
  ws->trace = nullptr;
  ws->trace_cap = 0;
  ws->maxdeg = g->maxdeg;
  ws->light = kInf;
  ws->qcap = V;
  ws->hcap = hcap;
  ws->srcs = nullptr;
  ws->nsrc = 0;
  ws->delta = 0;
  *cnt_out = cnt;
  return b.off;
}

size_t gdbi::sssp_workspace_bytes(const gdb_graph* g) {
  return sssp_layout(g, nullptr, nullptr, nullptr, nullptr);
}

// Mean and maximum usable weight, measured once per weight array.
static int weight_summary(gdb_ctx* c, gdb_graph* g) {
  if (g->wmean >= 0) return GDB_OK;
  unsigned long long* d = nullptr;
  unsigned long long* h = (unsigned long long*)pinned(c, 4096);
  if (!h) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, 24, c->stream));
  cudaError_t e = cudaMemsetAsync(d, 0, 24, c->stream);
  if (e == cudaSuccess && g->E) {
    k_weight_sum<<<4 * c->sm_count, 256, 0, c->stream>>>(g->w, g->E, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, 24, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return set_cuda_error(c, e, "weight summary");
  g->wmean = h[1] ? (double)h[0] / (double)h[1] : 1.0;
  g->wmax = (uint32_t)h[2];
  return GDB_OK;
}

// Automatic bucket width: 32 x mean weight / mean degree (the heuristic
// of Davidson et al.).
static int sssp_auto_delta(gdb_ctx* c, gdb_graph* g, uint32_t* delta) {
  *delta = 1;
  if (!g->w || g->E == 0) return GDB_OK;
  const int rc = weight_summary(c, g);
  if (rc) return rc;
  const double deg = (double)g->E / std::max<uint32_t>(g->V, 1);
  const double dl = 32.0 * g->wmean / std::max(deg, 1.0);
  *delta = (uint32_t)std::min(std::max(dl, 1.0), 1e9);
  return GDB_OK;
}

// Automatic width: the Davidson et al. width, a quarter of it when the
// light/heavy split is allowed and some arc weighs at least half of it.
// With heavy arcs relaxed once per vertex, narrow buckets pay: a bucket's
// near supersteps re-expand a vertex each time its distance improves, and
// on a power-law graph the first bucket holds most hubs.  R-MAT-22 with
// U[1,255] weights (the rule's width 134), 16 sources on lanes:
//   width 24: 16.4 ms, 28: 15.4, 32: 15.6, 40: 17.3, 48: 18.2, 67: 20.6,
//   96: 25.3, 134: 31.9 ms.
// Graphs whose weights stay below half the width (the 4096^2 grid: width
// 1,024, no split) keep the full width, where narrower buckets only add
// supersteps (grid SSSP 108 ms at 1,024, 131 at 512, 157 at 256).
static int sssp_auto_width(gdb_ctx* c, gdb_graph* g, uint32_t* delta) {
  int rc = sssp_auto_delta(c, g, delta);
  if (rc || c->opt.sssp_split < 0 || *delta < 2) return rc;
  if (c->opt.sssp_split == 1 || g->wmax >= *delta / 2) *delta = std::max<uint32_t>(*delta / 4, 1u);
  return GDB_OK;
}

// Light-arc bound of a near-far run of width `delta`: arcs of weight >=
// delta are deferred to the settle superstep when options.sssp_split asks
// for it (1) or, automatically (0), when the graph has such arcs; kInf =
// no split.
static int sssp_light_bound(gdb_ctx* c, gdb_graph* g, uint32_t delta, uint32_t* light) {
  *light = kInf;
  if (delta == 0 || c->opt.sssp_split < 0) return GDB_OK;
  if (c->opt.sssp_split == 0) {
    const int rc = weight_summary(c, g);
    if (rc) return rc;
    if (g->wmax < delta) return GDB_OK;
  }
  *light = std::min<uint32_t>(delta, kInf);
  return arc_split(c, g, *light);
}

// The views a run walks: the light half, the heavy half and its transpose
// under the split, the graph itself (three times) otherwise.
static void split_views(gdb_graph* g, uint32_t light, GraphView* gn, GraphView* gh, GraphView* gt) {
  if (light < kInf && g->split_l && g->split_bound == light) {
    *gn = g->split_l->view();
    *gh = g->split_h->view();
    *gt = g->split_t ? g->split_t->view() : *gh;  // a symmetric graph is its own transpose
  } else {
    *gn = *gh = *gt = g->view();
  }
}

// Schedule of one worklist SSSP run: the bucket width (0 = the
// label-correcting worklist), its light-arc bound and whether to run under
// graph relaunch.
//  * options.sssp_delta > 0: that width;
//  * learned: the selector's cheapest of worklist, near-far at the
//    automatic width, near-far at 4x that width and (where allowed) the
//    worklist under graph relaunch;
//  * adaptive: the automatic width;  * plain: the worklist;
// and under options.sssp_split the light-arc bound of a near-far width.
int gdbi::sssp_plan(gdb_ctx* c, gdb_graph* g, uint32_t nsrc, bool allow_relaunch, uint32_t* delta,
                    bool* relaunch, uint32_t* light) {
  *delta = 0;
  *relaunch = false;
  *light = kInf;
  int rc = GDB_OK;
  if (c->opt.sssp_delta) {
    *delta = c->opt.sssp_delta;
  } else if (c->opt.schedule == GDB_SCHED_ADAPTIVE) {
    rc = sssp_auto_width(c, g, delta);
  } else if (c->opt.schedule == GDB_SCHED_LEARNED) {
    if (c->h_mlp.empty()) return set_error(c, GDB_ERR_INVALID, "learned schedule without a selector");
    float x[kFeat], y[kOut];
    sssp_features(c, g, std::max<uint32_t>(nsrc, 1), x);
    mlp_host(c->h_mlp.data(), x, y);
    int best = kOutSsspPlain;
    for (int k = kOutSsspNearFar; k <= kOutSsspRelaunch; ++k) {
      if (k == kOutSsspRelaunch && !allow_relaunch) continue;
      if (y[k] < y[best]) best = k;
    }
    if (best == kOutSsspRelaunch) {
      *relaunch = true;
      return GDB_OK;
    }
    if (best != kOutSsspPlain) {
      uint32_t d = 1;
      rc = sssp_auto_width(c, g, &d);
      *delta = best == kOutSsspNearFarWide ? (uint32_t)std::min<uint64_t>(4ull * d, 1000000000ull) : d;
    }
  }
  if (rc) return rc;
  return sssp_light_bound(c, g, *delta, light);
}

// Settle direction of a run (see SsspWs::settle): only the split has
// settle supersteps; the learned schedule hands them to the selector.
static int settle_of(const gdb_ctx* c, uint32_t light, int force) {
  if (light >= kInf) return kSettleRule;
  if (force >= 0) return force;
  return c->opt.schedule == GDB_SCHED_LEARNED && c->d_mlp ? kSettleLearned : kSettleRule;
}

int gdbi::sssp_enqueue(gdb_ctx* c, gdb_graph* g, void* wsbase, const uint32_t* d_srcs, uint32_t nsrc,
                       uint32_t* d_dist, cudaStream_t stream, const gdb::DiscoveryArgs& proto,
                       uint32_t delta, uint32_t light) {
  if (!g->w) return set_error(c, GDB_ERR_INVALID, "SSSP needs weights");
  SsspWs ws;
  char* cnt = nullptr;
  sssp_layout(g, (char*)wsbase, d_dist, &ws, &cnt);
  ws.srcs = d_srcs;
  ws.nsrc = nsrc;
  ws.delta = delta;
  // a plan whose partition was dropped since (new weights) runs unsplit
  ws.light = delta && light < kInf && g->split_l && g->split_bound == light ? light : kInf;
  GraphView GN, GH, GT;
  split_views(g, ws.light, &GN, &GH, &GT);
  ws.settle = settle_of(c, ws.light, -1);
  ws.mlp = c->d_mlp;
  GDB_CUDA(c, cudaMemsetAsync(cnt, 0, 512, stream));
  Shape s;
  auto kx = ws.settle == kSettleRule ? k_sssp_xf : k_sssp_xf_sel;
  int rc = persistent_shape(c, (const void*)kx, c->opt.block_size, 0, &s, false);
  if (rc) return rc;
  DiscoveryArgs a = proto;
  a.expected = std::min(s.grid, s.fit);
  kx<<<s.grid, c->opt.block_size, 0, stream>>>(a, GN, GH, GT, ws, 0u);
  GDB_CUDA(c, cudaGetLastError());
  return GDB_OK;
}

// force_settle >= 0: a fixed settle direction (trace runs), recording up to
// trace_cap settle supersteps in d_trace.
static int sssp_run(gdb_ctx* c, gdb_graph* g, uint32_t src, const uint32_t* d_srcs, uint32_t nsrc,
                    uint32_t* d_dist, int force_settle = -1, gdb_level_trace* d_trace = nullptr,
                    uint32_t trace_cap = 0) {
  if (!graph_ok(c, g) || !d_dist || (nsrc && !d_srcs)) return GDB_ERR_INVALID;
  if (!nsrc && src >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  if (!g->w) return set_error(c, GDB_ERR_INVALID, "SSSP needs weights");
  // relaunched supersteps run the plain worklist
  const bool relaunched = c->opt.barrier == GDB_BARRIER_RELAUNCH_GRAPH || c->opt.barrier == GDB_BARRIER_RELAUNCH;
  if (nsrc && relaunched)
    return set_error(c, GDB_ERR_UNSUPPORTED, "multi-source SSSP needs a persistent barrier");
  uint32_t delta = 0, light = kInf;
  bool relaunch = false;
  int rc = relaunched ? GDB_OK : sssp_plan(c, g, nsrc ? nsrc : 1, nsrc == 0, &delta, &relaunch, &light);
  if (rc) return rc;
  char* base = (char*)workspace(c, sssp_layout(g, nullptr, nullptr, nullptr, nullptr));
  if (!base) return GDB_ERR_OOM;
  SsspWs ws;
  char* cnt = nullptr;
  sssp_layout(g, base, d_dist, &ws, &cnt);
  ws.srcs = d_srcs;
  ws.nsrc = nsrc;
  ws.delta = delta;
  // the split lives in the persistent kernels only (graph relaunch runs
  // the plain worklist)
  ws.light = relaunch ? kInf : light;
  const int kind = relaunch ? GDB_BARRIER_RELAUNCH_GRAPH : c->opt.barrier;
  const bool xf = kind == GDB_BARRIER_XF || kind == GDB_BARRIER_XF_FIXED;
  ws.settle = xf ? settle_of(c, ws.light, force_settle) : kSettleRule;
  ws.mlp = c->d_mlp;
  ws.trace = d_trace;
  ws.trace_cap = trace_cap;
  const GraphView G = g->view();
  GraphView GN, GH, GT;
  split_views(g, ws.light, &GN, &GH, &GT);
  GDB_CUDA(c, cudaMemsetAsync(cnt, 0, 512, c->stream));
  const int block = c->opt.block_size;
  c->last = gdb_run_stats{};
  if (xf) {
    Shape s;
    auto kx = ws.settle == kSettleRule ? k_sssp_xf : k_sssp_xf_sel;
    rc = persistent_shape(c, (const void*)kx, block, 0, &s, kind == GDB_BARRIER_XF);
    if (rc) return rc;
    DiscoveryArgs a = discovery_args(c, s);
    GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    kx<<<s.grid, block, 0, c->stream>>>(a, GN, GH, GT, ws, src);
    GDB_CUDA(c, cudaGetLastError());
    GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    rc = finish_run(c);
    if (rc) return rc;
    int n = 0;
    read_participating(c, &n);
    c->last.participating = n;
    c->last.launched = s.grid;
  } else if (kind == GDB_BARRIER_GRID_SYNC) {
    int occ = 0;
    GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sssp_grid, block, 0));
    int grid = occ * c->sm_count;
    if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
    GraphView Gc = GN, GHc = GH, GTc = GT;
    SsspWs wsc = ws;
    uint32_t srcc = src;
    void* args[] = {(void*)&Gc, (void*)&GHc, (void*)&GTc, (void*)&wsc, (void*)&srcc};
    GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    GDB_CUDA(c, cudaLaunchCooperativeKernel((const void*)k_sssp_grid, grid, block, args, 0, c->stream));
    GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    GDB_CUDA(c, cudaStreamSynchronize(c->stream));
    c->last.participating = grid;
    c->last.launched = grid;
  } else if (kind == GDB_BARRIER_RELAUNCH_GRAPH) {
    int occ = 0;
    GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sssp_glevel, block, 0));
    int grid = occ * c->sm_count;
    if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
    uint32_t* ctl = (uint32_t*)(cnt + 192);  // [0] superstep, [1] CTAs done, [2] host loop, [3] stop
    GDB_CUDA(c, cudaMemsetAsync(ctl, 0, 16, c->stream));
    rc = graph_while_run(c, (const void*)k_sssp_init, grid, block, G, ws, src,
                         (const void*)k_sssp_glevel, ctl);
    if (rc) return rc;
    c->last.participating = grid;
    c->last.launched = grid;
  } else if (kind == GDB_BARRIER_RELAUNCH) {
    // the reference's host loop: one launch per superstep, the stop word
    // read back after each
    int occ = 0;
    GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sssp_glevel, block, 0));
    int grid = occ * c->sm_count;
    if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
    uint32_t* ctl = (uint32_t*)(cnt + 192);
    uint32_t* h = (uint32_t*)pinned(c, 64);
    if (!h) return GDB_ERR_OOM;
    GDB_CUDA(c, cudaMemsetAsync(ctl, 0, 16, c->stream));
    GDB_CUDA(c, cudaMemsetAsync(ctl + 2, 1, 1, c->stream));  // ctl[2] = 1: host loop
    GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    k_sssp_init<<<grid, block, 0, c->stream>>>(G, ws, src);
    GDB_CUDA(c, cudaGetLastError());
    uint32_t launches = 1;
    for (;;) {
      k_sssp_glevel<<<grid, block, 0, c->stream>>>(G, ws, ctl, 0);
      ++launches;
      GDB_CUDA(c, cudaMemcpyAsync(h, ctl + 3, 4, cudaMemcpyDeviceToHost, c->stream));
      GDB_CUDA(c, cudaStreamSynchronize(c->stream));
      if (h[0]) break;
    }
    GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    GDB_CUDA(c, cudaStreamSynchronize(c->stream));
    c->last.participating = grid;
    c->last.launched = grid;
    c->last.launches = launches;
  } else {
    return set_error(c, GDB_ERR_UNSUPPORTED, "barrier kind not available for SSSP");
  }
  if (kind == GDB_BARRIER_XF || kind == GDB_BARRIER_XF_FIXED || kind == GDB_BARRIER_GRID_SYNC)
    c->last.launches = 1;
  unsigned long long* hs = (unsigned long long*)pinned(c, 512);
  if (!hs) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hs, cnt, 512, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (*(int*)((char*)hs + 160)) return set_error(c, GDB_ERR_CAPACITY, "SSSP queue overflow");
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last.kernel_ms = ms;
  c->last.edges_processed = hs[0];
  c->last.supersteps = (uint32_t)hs[1];
  if (kind == GDB_BARRIER_RELAUNCH_GRAPH) c->last.launches = 1 + c->last.supersteps;  // init + supersteps
  c->last.phases = (uint32_t)hs[2];
  c->last.sssp_delta = delta;
  c->last.sssp_light = ws.light < kInf ? ws.light : 0u;
  return GDB_OK;
}

static int jacobi_run(gdb_ctx* c, gdb_graph* g, uint32_t src, int32_t* d_cost) {
  if (!graph_ok(c, g) || !d_cost) return GDB_ERR_INVALID;
  if (src >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  if (!g->w) return set_error(c, GDB_ERR_INVALID, "SSSP needs weights");
  const int kind = c->opt.barrier;
  const bool relaunch = kind == GDB_BARRIER_RELAUNCH || kind == GDB_BARRIER_RELAUNCH_GRAPH;
  if (kind != GDB_BARRIER_XF && kind != GDB_BARRIER_XF_FIXED && !relaunch)
    return set_error(c, GDB_ERR_UNSUPPORTED, "Jacobi SSSP runs on the XF barrier or relaunched");
  Bump b;
  const size_t o_x = b.take((size_t)g->V * 4);
  const size_t o_cnt = b.take(256);
  const size_t o_ctl = b.take(sizeof(StepCtl));
  char* base = (char*)workspace(c, b.off);
  if (!base) return GDB_ERR_OOM;
  JacobiWs ws;
  ws.x[0] = d_cost;
  ws.x[1] = (int32_t*)(base + o_x);
  char* cnt = base + o_cnt;
  ws.stats = (unsigned long long*)cnt;
  ws.cursor = (uint32_t*)(cnt + 64);
  ws.hcursor = (uint32_t*)(cnt + 80);
  ws.changed = (uint32_t*)(cnt + 96);
  const GraphView G = g->view();
  const int block = c->opt.block_size;
  c->last = gdb_run_stats{};
  Shape s;
  int rc = GDB_OK;
  if (relaunch) {
    int grid = 0;
    if ((rc = step_grid(c, (const void*)k_jacobi_rl_step, block, &grid))) return rc;
    StepCtl first{};
    // at most num_rows - 1 iterations (sssp_kernel.cl:185)
    rc = step_run(c, kind, (const void*)k_jacobi_rl_init, (const void*)k_jacobi_rl_step, grid, block,
                  (StepCtl*)(base + o_ctl), first, (unsigned long long)g->V + 1, g->V >= 2, G, ws, src);
    if (rc) return rc;
    s.grid = grid;
  } else {
    rc = persistent_shape(c, (const void*)k_jacobi_xf, block, 0, &s, kind == GDB_BARRIER_XF);
    if (rc) return rc;
    DiscoveryArgs a = discovery_args(c, s);
    GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    k_jacobi_xf<<<s.grid, block, 0, c->stream>>>(a, G, ws, src);
    GDB_CUDA(c, cudaGetLastError());
    GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    rc = finish_run(c);
    if (rc) return rc;
  }
  const uint32_t launches = relaunch ? c->last.launches : 1;
  unsigned long long* hs = (unsigned long long*)pinned(c, 256);
  if (!hs) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hs, cnt, 64, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  const uint32_t k = (uint32_t)hs[1];
  if (k >= 1 && ((k - 1) & 1)) {
    GDB_CUDA(c, cudaMemcpyAsync(d_cost, ws.x[1], (size_t)g->V * 4, cudaMemcpyDeviceToDevice, c->stream));
  }
  GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  int n = s.grid;
  if (!relaunch) read_participating(c, &n);
  c->last.participating = n;
  c->last.launched = s.grid;
  c->last.launches = launches;
  c->last.kernel_ms = ms;
  c->last.edges_processed = hs[0];
  c->last.supersteps = k;
  return GDB_OK;
}

extern "C" {

int gdb_sssp_jacobi_device(gdb_ctx* c, gdb_graph* g, uint32_t src, int32_t* d_cost) {
  return jacobi_run(c, g, src, d_cost);
}

int gdb_sssp_jacobi(gdb_ctx* c, gdb_graph* g, uint32_t src, int32_t* cost) {
  if (!graph_ok(c, g) || !cost) return GDB_ERR_INVALID;
  int32_t* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, (size_t)g->V * 4, c->stream));
  int rc = jacobi_run(c, g, src, d);
  if (rc == GDB_OK) {
    cudaError_t e = cudaMemcpyAsync(cost, d, (size_t)g->V * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "cost read-back");
  }
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

int gdb_sssp_device(gdb_ctx* c, gdb_graph* g, uint32_t src, uint32_t* d_dist) {
  return sssp_run(c, g, src, nullptr, 0, d_dist);
}

int gdb_sssp_multi_device(gdb_ctx* c, gdb_graph* g, const uint32_t* d_sources, uint32_t nsrc,
                          uint32_t* d_dist) {
  if (nsrc == 0) return GDB_ERR_INVALID;
  return sssp_run(c, g, 0, d_sources, nsrc, d_dist);
}

int gdb_sssp_multi(gdb_ctx* c, gdb_graph* g, const uint32_t* sources, uint32_t nsrc, uint32_t* dist) {
  if (!graph_ok(c, g) || !dist || !sources || nsrc == 0) return GDB_ERR_INVALID;
  for (uint32_t i = 0; i < nsrc; ++i)
    if (sources[i] >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  const size_t nb = (size_t)g->V * 4;
  char* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, nb + (size_t)nsrc * 4, c->stream));
  cudaError_t e = cudaMemcpyAsync(d + nb, sources, (size_t)nsrc * 4, cudaMemcpyHostToDevice, c->stream);
  int rc = e == cudaSuccess ? sssp_run(c, g, 0, (const uint32_t*)(d + nb), nsrc, (uint32_t*)d)
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

int gdb_sssp_sources_device(gdb_ctx* c, gdb_graph* g, const uint32_t* d_sources, uint32_t n,
                            uint32_t* d_dist) {
  if (!graph_ok(c, g) || !d_sources || !d_dist || n == 0) return GDB_ERR_INVALID;
  if (!g->w) return set_error(c, GDB_ERR_INVALID, "SSSP needs weights");
  const size_t V = g->V;
  if (c->opt.barrier != GDB_BARRIER_XF && c->opt.barrier != GDB_BARRIER_XF_FIXED) {
    for (uint32_t i = 0; i < n; ++i) {
      const int rc = sssp_run(c, g, 0, d_sources + i, 1, d_dist + i * V);
      if (rc) return rc;
    }
    return GDB_OK;
  }
  uint32_t delta = 0, light = kInf;
  bool relaunch = false;
  int rc = sssp_plan(c, g, 1, false, &delta, &relaunch, &light);
  if (rc) return rc;
  int occ = 0;
  GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sssp_xf, c->opt.block_size, 0));
  rc = run_on_lanes(c, n, kSsspLanes, true, sssp_workspace_bytes(g), occ * c->sm_count,
                    [&](gdb_lane& L, uint32_t i) {
    return sssp_enqueue(c, g, L.ws, d_sources + i, 1, d_dist + i * V, L.stream, lane_args(c, L),
                        delta, light);
  });
  c->last.sssp_delta = delta;
  c->last.sssp_light = delta && light < kInf ? light : 0u;
  return rc;
}

int gdb_sssp_sources(gdb_ctx* c, gdb_graph* g, const uint32_t* sources, uint32_t n, uint32_t* dist) {
  if (!graph_ok(c, g) || !dist || !sources || n == 0) return GDB_ERR_INVALID;
  for (uint32_t i = 0; i < n; ++i)
    if (sources[i] >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  const size_t nb = (size_t)g->V * 4 * n;
  char* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, nb + (size_t)n * 4, c->stream));
  cudaError_t e = cudaMemcpyAsync(d + nb, sources, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
  int rc = e == cudaSuccess ? gdb_sssp_sources_device(c, g, (const uint32_t*)(d + nb), n, (uint32_t*)d)
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

int gdb_sssp_trace(gdb_ctx* c, gdb_graph* g, uint32_t src, int mode, uint32_t* dist,
                   gdb_level_trace* trace, uint32_t cap, uint32_t* settles) {
  if (!graph_ok(c, g) || mode < 0 || mode > 2 || (cap && !trace)) return GDB_ERR_INVALID;
  if (src >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  if (c->opt.barrier != GDB_BARRIER_XF && c->opt.barrier != GDB_BARRIER_XF_FIXED)
    return set_error(c, GDB_ERR_UNSUPPORTED, "settle traces need the XF barrier");
  if (mode == 2 && !c->d_mlp) return set_error(c, GDB_ERR_INVALID, "no selector loaded");
  const int force = mode == 0 ? kSettlePush : mode == 1 ? kSettlePull : kSettleLearned;
  const size_t nb = (size_t)g->V * 4, tb = (size_t)std::max<uint32_t>(cap, 1) * sizeof(gdb_level_trace);
  char* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, nb + tb, c->stream));
  cudaError_t e = cudaMemsetAsync(d + nb, 0, tb, c->stream);
  int rc = e == cudaSuccess ? sssp_run(c, g, src, nullptr, 0, (uint32_t*)d, force, (gdb_level_trace*)(d + nb), cap)
                            : set_cuda_error(c, e, "trace buffer");
  uint32_t n = 0;
  if (rc == GDB_OK) {
    if (dist) e = cudaMemcpyAsync(dist, d, nb, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && cap)
      e = cudaMemcpyAsync(trace, d + nb, (size_t)cap * sizeof(gdb_level_trace), cudaMemcpyDeviceToHost,
                          c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "trace read-back");
    // settle records: those with a duration (the trace may be shorter than the run)
    for (uint32_t i = 0; rc == GDB_OK && i < cap && trace[i].us > 0.f; ++i) ++n;
  }
  if (settles) *settles = n;
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

int gdb_sssp(gdb_ctx* c, gdb_graph* g, uint32_t src, uint32_t* dist) {
  if (!graph_ok(c, g) || !dist) return GDB_ERR_INVALID;
  uint32_t* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, (size_t)g->V * 4, c->stream));
  int rc = sssp_run(c, g, src, nullptr, 0, d);
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
