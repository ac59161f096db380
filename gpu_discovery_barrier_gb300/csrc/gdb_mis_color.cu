// Maximal independent set and greedy colouring with Pannotia semantics.
//
// MIS (mega_kernel, pannotia/graph_app/mis/kernel/mis_kernel.cl:220-337):
// per round every undecided vertex takes the minimum priority over its
// undecided neighbours (mis1, :245-270); undecided strict local minima join
// the set, s = 2, and mark their undecided neighbours decided (mis2,
// :277-312).  The reference stages neighbour marks in cu[] and commits them
// in a third barrier interval (mis3, :322-330); here the marks go straight
// into the state array -- two winners are never adjacent, so no winner test
// can see a mark of the same round -- and a round needs two barriers.
//
// Colouring (mega_kernel, pannotia/graph_app/color/kernel/color_kernel.cl:159-252):
// per round every uncoloured vertex takes the maximum priority over its
// uncoloured neighbours -- a degree-1 vertex ignores its only neighbour
// (start != end - 1, :204) -- then the uncoloured vertices above it take
// the round's colour; stop after a round in which no vertex saw an
// uncoloured neighbour.  Colours start at 1.
//
// Priorities are compared as floats through an order-preserving uint32
// key, so shared-memory atomicMin/atomicMax give the per-vertex extremum.
#include <algorithm>

#include "gdb_internal.h"
#include "gdb_relaunch.cuh"

namespace {

using namespace gdb;

constexpr float kMisBig = 99999999.0f;  // BIGNUM, mis_kernel.cl:68

struct MisWs {
  int32_t* state;       // -1 undecided, -2 decided
  uint32_t* ukey;       // the priority key while undecided, kMisGone once decided
  int32_t* s;           // output: 2 in the set, 0 otherwise
  uint32_t* mn;         // light vertices: key of the min undecided neighbour priority
  uint32_t* hmn[2];     // heavy vertices, by heavy index, double-buffered by round
  const float* prio;
  uint32_t* cursor;     // [3]
  uint32_t* hcursor;    // [3]
  uint32_t* flag;       // [3] some vertex undecided
  uint32_t* won;        // [3] some vertex joined the set (mis2 supersteps)
  int* stuck;           // set when a round chose no vertex (see mis_body)
  unsigned long long* stats;  // [0] arcs, [1] rounds
};

constexpr uint32_t kMisNone = 0xFFFFFFFFu;  // no arc in this lane's step
// ukey of a decided vertex: above every key mis1 can take as a minimum
// (BIGNUM's key and all finite priorities), so a decided neighbour never
// lowers one, and mis1 needs one load per neighbour instead of the state
// and then the priority
constexpr uint32_t kMisGone = 0xFFFFFFFFu;

// A priority's key: fkey's order, with every NaN, of either sign, at
// kMisGone -- above all numbers, so that a NaN priority never wins and
// never lowers a neighbour's minimum, as the reference's comparisons with
// NaN are all false (fkey alone would put a NaN with its sign bit set
// below every number).
__device__ __forceinline__ uint32_t mis_key(float f) { return isnan(f) ? kMisGone : fkey(f); }

// mis_kernel.cl:78-93 (init), run by every thread of the grid.
__device__ __forceinline__ void mis_init(const GraphView& G, const Warps& W, const MisWs& ws, bool leader) {
  const uint32_t big = fkey(kMisBig);
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
    ws.state[v] = -1;
    ws.s[v] = 0;
    ws.ukey[v] = mis_key(__ldg(&ws.prio[v]));
  }
  for (uint32_t h = W.gthread; h < G.nheavy; h += W.nthreads) ws.hmn[0][h] = ws.hmn[1][h] = big;
  if (leader) {
    for (int i = 0; i < 3; ++i) ws.cursor[i] = ws.hcursor[i] = ws.flag[i] = ws.won[i] = 0;
    *ws.stuck = 0;
    ws.stats[0] = ws.stats[1] = 0;
  }
}

// mis1 of round r (superstep t): every undecided vertex takes the minimum
// priority key over its undecided neighbours; flag[t % 3] records whether
// any vertex was still undecided.  Every thread of the grid calls it.
__device__ __forceinline__ void mis_phase1(const GraphView& G, const MisWs& ws, uint32_t r, uint32_t t,
                                           uint32_t* my, bool leader, unsigned long long& arcs) {
  const int lane = lane_id();
  const uint32_t big = fkey(kMisBig);
  // flag[t % 3] is read after this superstep's barrier: clear the slot
  // of superstep t - 2
  const int cur = t % 3, old = (t + 1) % 3;
  if (leader) ws.cursor[old] = ws.hcursor[old] = ws.flag[old] = 0;
  bool undecided_seen = false;
  // four 32-arc steps at once: the column and key loads of the four are
  // in flight together
  sweep_light4(
      G, &ws.cursor[cur],
      [&](uint32_t v, bool in_range) {
        const bool und = in_range && ld_cg(&ws.state[v]) == -1;
        my[lane] = big;
        undecided_seen |= und;
        return und;
      },
      [&](const bool* valid, const int* owner, const uint32_t* arc) {
        uint32_t u[4], k[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          u[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
          arcs += valid[j];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) k[j] = valid[j] ? ld_cg(&ws.ukey[u[j]]) : kMisGone;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (k[j] < my[owner[j]]) atomicMin(&my[owner[j]], k[j]);
      },
      [&](uint32_t v, bool act) {
        if (act) ws.mn[v] = my[lane];
      });
  uint32_t* hmn = pick(ws.hmn, r);
  sweep_heavy(G, &ws.hcursor[cur], [&](uint32_t v, uint32_t h, uint32_t, uint32_t b, uint32_t e) {
    // a heavy winner's own state is settled here (see mis2)
    if (ld_cg(&ws.s[v]) == 2) {
      if (lane == 0) {
        ws.state[v] = -2;
        ws.ukey[v] = kMisGone;
      }
      return;
    }
    if (ld_cg(&ws.state[v]) != -1) return;
    undecided_seen = true;
    uint32_t m = big;
    // a chunk (kChunk = 128 arcs) as four steps with their loads in flight
    uint32_t u[4], k[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t a = b + 32 * j + lane;
      u[j] = a < e ? __ldg(&G.col[a]) : kMisNone;
      arcs += a < e;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) k[j] = u[j] != kMisNone ? ld_cg(&ws.ukey[u[j]]) : kMisGone;
#pragma unroll
    for (int j = 0; j < 4; ++j) m = min(m, k[j]);
    m = warp_min_u32(m);
    if (lane == 0 && m < big) atomicMin(&hmn[h], m);
  });
  cta_or(undecided_seen, &ws.flag[cur], 1u);
}

// mis2 of round r (superstep t): strict local minima join the set and
// decide their neighbours.  Every thread of the grid calls it.
__device__ __forceinline__ void mis_phase2(const GraphView& G, const Warps& W, const MisWs& ws, uint32_t r,
                                           uint32_t t, bool leader, unsigned long long& arcs) {
  const int lane = lane_id();
  const uint32_t big = fkey(kMisBig);
  // flag[t % 3] and won[t % 3] are read after this superstep's barrier:
  // clear the slots of superstep t - 2
  const int cur = t % 3, old = (t + 1) % 3;
  if (leader) ws.cursor[old] = ws.hcursor[old] = ws.flag[old] = ws.won[old] = 0;
  bool any_win = false;
  // next round's heavy minima start from BIGNUM
  for (uint32_t h = W.gthread; h < G.nheavy; h += W.nthreads) pick(ws.hmn, r + 1)[h] = big;
  sweep_light4(
      G, &ws.cursor[cur],
      [&](uint32_t v, bool in_range) {
        bool win = false;
        if (in_range && ld_cg(&ws.state[v]) == -1 && mis_key(__ldg(&ws.prio[v])) < ws.mn[v]) {
          win = true;
          any_win = true;
          ws.s[v] = 2;
          ws.state[v] = -2;
          ws.ukey[v] = kMisGone;
        }
        return win;
      },
      [&](const bool* valid, const int*, const uint32_t* arc) {
        uint32_t u[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          u[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
          arcs += valid[j];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (valid[j] && ld_cg(&ws.state[u[j]]) == -1) {
            ws.state[u[j]] = -2;
            ws.ukey[u[j]] = kMisGone;
          }
      },
      [](uint32_t, bool) {});
  const uint32_t* hmn = pick(ws.hmn, r);
  // A heavy winner is split over chunks: its own state stays -1 here so
  // every chunk sees the same test; s = 2 marks it and mis1 of the next
  // round settles its state (all its neighbours are decided by then, so
  // nobody reads it in between).
  sweep_heavy(G, &ws.hcursor[cur], [&](uint32_t v, uint32_t h, uint32_t, uint32_t b, uint32_t e) {
    if (ld_cg(&ws.state[v]) != -1) return;
    if (!(mis_key(__ldg(&ws.prio[v])) < ld_cg(&hmn[h]))) return;
    any_win = true;
    if (lane == 0) ws.s[v] = 2;
    uint32_t u[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t a = b + 32 * j + lane;
      u[j] = a < e ? __ldg(&G.col[a]) : kMisNone;
      arcs += a < e;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (u[j] != kMisNone && ld_cg(&ws.state[u[j]]) == -1) {
        ws.state[u[j]] = -2;
        ws.ukey[u[j]] = kMisGone;
      }
  });
  cta_or(any_win, &ws.won[cur], 1u);
}

template <class Sync>
__device__ __forceinline__ void mis_body(Sync& s, const GraphView& G, const MisWs& ws, uint32_t* smem) {
  const Warps W = warps_of(s.id(), s.P());
  const bool leader = s.id() == 0 && threadIdx.x == 0;
  uint32_t* my = smem + (threadIdx.x & ~31u);
  mis_init(G, W, ws, leader);
  if (!s.sync()) return;
  unsigned long long arcs = 0;
  uint32_t r = 0;
  uint32_t t = 0;  // cursor slot counter: two sweeps per round
  // A round in which no vertex joins the set changes nothing, so every
  // later round would repeat it: adjacent vertices of equal priority, NaN
  // priorities and priorities of BIGNUM and above never win.  The
  // reference loops forever then; here the kernel stops at that round and
  // the host reports it.  A round that does choose a vertex decides at
  // least that one, so V rounds always suffice: the bound below holds the
  // loop to them whatever happens.
  for (; r <= G.V; ++r) {
    mis_phase1(G, ws, r, t, my, leader, arcs);
    if (!s.sync()) return;
    const int cur = t % 3;
    ++t;
    if (cta_words<1>([&](unsigned long long* w) { w[0] = ld_cg(&ws.flag[cur]); })[0] == 0) break;
    mis_phase2(G, W, ws, r, t, leader, arcs);
    if (!s.sync()) return;
    const int cur2 = t % 3;
    ++t;
    if (cta_words<1>([&](unsigned long long* w) { w[0] = ld_cg(&ws.won[cur2]); })[0] == 0) {
      if (leader) *ws.stuck = 1;
      break;
    }
  }
  if (r > G.V && leader) *ws.stuck = 1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) arcs += __shfl_xor_sync(kFull, arcs, o);
  if (lane_id() == 0 && arcs) atomicAdd(&ws.stats[0], arcs);
  if (leader) ws.stats[1] = r + 1;
}

__global__ void __launch_bounds__(512, 3) k_mis_xf(DiscoveryArgs a, GraphView G, MisWs ws) {
  __shared__ LocalCtx l;
  __shared__ uint32_t smem[1024];
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  mis_body(s, G, ws, smem);
}

// Relaunch form (mis.cpp:314-364: one launch per phase, the stop flag read
// back after each): control state s[0] = round, s[1] = superstep, s[2] =
// phase (1: mis1, 2: mis2).
__global__ void k_mis_rl_init(GraphView G, MisWs ws) {
  mis_init(G, warps_of(blockIdx.x, gridDim.x), ws, blockIdx.x == 0 && threadIdx.x == 0);
}

__global__ void __launch_bounds__(512, 3) k_mis_rl_step(GraphView G, MisWs ws, StepCtl* ctl,
                                                       cudaGraphConditionalHandle cond) {
  __shared__ uint32_t smem[1024];
  const StepCtl& st0 = step_state(ctl);
  const uint32_t r = st0.s[0], t = st0.s[1], phase = st0.s[2];
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long arcs = 0;
  if (phase == 1)
    mis_phase1(G, ws, r, t, smem + (threadIdx.x & ~31u), leader, arcs);
  else
    mis_phase2(G, warps_of(blockIdx.x, gridDim.x), ws, r, t, leader, arcs);
  arcs = warp_add_u64(arcs);
  if (lane_id() == 0 && arcs) atomicAdd(&ws.stats[0], arcs);
  step_end(ctl, cond, [&](StepCtl& st) {
    st.s[1] = t + 1;
    if (phase == 1) {
      if (__ldcg(&ws.flag[t % 3]) == 0) {
        ws.stats[1] = r + 1;
        return false;
      }
      st.s[2] = 2;
    } else {
      if (__ldcg(&ws.won[t % 3]) == 0) {
        // no vertex joined the set: every later round would repeat this one
        *ws.stuck = 1;
        ws.stats[1] = r + 1;
        return false;
      }
      st.s[0] = r + 1;
      st.s[2] = 1;
    }
    return true;
  });
}

// ------------------------------------------------------------- colouring
//
// The round structure of the reference colours v in the first round after
// all of its higher-priority neighbours are coloured: colour(v) = 1 + the
// largest colour among them (0 if none), and a degree-1 vertex takes 1.
// Re-scanning every uncoloured vertex's arcs each round (the reference's
// O(E x rounds), thousands of rounds on R-MAT) is replaced by peeling that
// priority DAG: every vertex counts the neighbours it waits for; the
// vertices coloured in round r walk their arcs once and count down their
// lower-priority neighbours, and a counter reaching zero puts that vertex
// in round r+1.  One barrier per round, every arc touched twice in total,
// the same colours.  Neighbours of equal priority wait for each other, so
// -- as in the reference, which never terminates then -- they stay
// uncoloured; the host reports that as an error.

struct ColorWs {
  int32_t* color;
  uint32_t* cnt;       // neighbours still to be coloured before this vertex
  uint32_t* wcol;      // from row[v]: the wcnt[v] neighbours that wait for v (the count pass)
  uint32_t* wcnt;
  const float* prio;
  uint2* q[2];                 // light vertices as their arc ranges {begin, end}
  uint4* hc[2];                // heavy chunks as {vertex, first arc, end arc, chunk}
  uint32_t* qcount;            // [3]
  unsigned long long* hcount;  // [3]
  uint32_t* cursor;            // [3]
  uint32_t* hcursor;           // [3]
  int* overflow;
  unsigned long long* stats;   // [0] arcs, [1] rounds, [2] coloured vertices
  uint32_t qcap, hcap;
};

// u waits for v when u looks at its neighbours (degree != 1) and v's
// priority is not below u's.  The count pass packs, for every vertex v,
// the neighbours waiting for v at the start of v's arc range (wcol from
// row[v], wcnt[v] of them), so a round walks only arcs that count down:
// half of the arcs, one load each, and a hub's entry is cut into chunks of
// its waiting arcs.  A vertex is a heavy (chunked) entry when more than
// kHeavyDeg neighbours wait for it.

// The colouring's frontier entries carry arc ranges, so a round's consumer
// needs no row load: the producer loads the rows of every vertex it counts
// down, in flight with the count-down itself.  Light entries are staged per
// warp in shared memory and leave 32 at a time; a heavy vertex's chunks are
// reserved with one packed atomic per warp step.
struct RangeStage {
  uint2* buf;    // this warp's 64 slots
  uint2* q;
  uint32_t* count;
  uint32_t cap;
  int* overflow;
  uint32_t n = 0;
  __device__ __forceinline__ void out(uint2 x, uint32_t m) {
    const int lane = lane_id();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(count, m);
    base = __shfl_sync(kFull, base, 0);
    if ((uint32_t)lane < m) {
      if (base + lane < cap) q[base + lane] = x;
      else atomicExch(overflow, 1);
    }
  }
  __device__ __forceinline__ void add(bool want, uint2 x) {
    const unsigned m = __ballot_sync(kFull, want);
    if (!m) return;
    const int lane = lane_id();
    if (want) buf[n + __popc(m & lanemask_lt())] = x;
    n += __popc(m);
    if (n >= 32) {
      __syncwarp();
      const uint2 y = buf[lane];
      const uint32_t r = n - 32;
      const uint2 z = (uint32_t)lane < r ? buf[32 + lane] : make_uint2(0u, 0u);
      __syncwarp();
      if ((uint32_t)lane < r) buf[lane] = z;
      __syncwarp();
      out(y, 32);
      n = r;
    }
  }
  __device__ __forceinline__ void flush() {
    __syncwarp();
    if (n) out((uint32_t)lane_id() < n ? buf[lane_id()] : make_uint2(0u, 0u), n);
    n = 0;
  }
};

// Push the lanes' ready vertices u with arc ranges [rb, re): light ones
// (degree <= kHeavyDeg) staged, heavy ones as chunk entries.
__device__ __forceinline__ void push_ranges(const ColorWs& ws, RangeStage& st, uint4* hc,
                                            unsigned long long* hcount, bool ready, bool heavy,
                                            uint32_t u, uint32_t rb, uint32_t re) {
  st.add(ready && !heavy && re > rb, make_uint2(rb, re));
  const bool hv = ready && heavy;
  const unsigned hm = __ballot_sync(kFull, hv);
  if (!hm) return;
  const int lane = lane_id();
  const uint32_t nch = hv ? chunks_of(re - rb) : 0u;
  uint32_t inc = nch;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  const uint32_t total = __shfl_sync(kFull, inc, 31);
  const int leader = __ffs(hm) - 1;
  unsigned long long old = 0;
  if (lane == leader) old = atomicAdd(hcount, ((unsigned long long)__popc(hm) << 32) | total);
  old = __shfl_sync(kFull, old, leader);
  const uint32_t cbase = (uint32_t)old;
  if (cbase + total > ws.hcap) {
    if (lane == leader) atomicExch(ws.overflow, 1);
    return;
  }
  const uint32_t first = cbase + inc - nch;
  for (unsigned m = hm; m; m &= m - 1) {
    const int l = __ffs(m) - 1;
    const uint32_t v = __shfl_sync(kFull, u, l), n = __shfl_sync(kFull, nch, l);
    const uint32_t f = __shfl_sync(kFull, first, l), b0 = __shfl_sync(kFull, rb, l),
                   e0 = __shfl_sync(kFull, re, l);
    for (uint32_t j = lane; j < n; j += 32)
      hc[f + j] = make_uint4(v, b0 + j * kChunk, min(e0, b0 + (j + 1) * kChunk), j);
  }
}

// Superstep 0: every colour -1, the heavy vertices' counters 0.
__device__ __forceinline__ void color_init(const GraphView& G, const Warps& W, const ColorWs& ws) {
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
    ws.color[v] = -1;
    if (is_heavy(G, v)) ws.cnt[v] = ws.wcnt[v] = 0;
  }
}

// Superstep 1: count the neighbours each vertex waits for, and pack the
// neighbours that wait for it (my / wmy: per-lane counters of a warp).
__device__ __forceinline__ void color_count(const GraphView& G, const ColorWs& ws, uint32_t* my,
                                            uint32_t* wmy, unsigned long long& arcs) {
  const int lane = lane_id();
  {
    float pv_lane = 0.f;
    bool looks_lane = false;
    uint32_t rv_lane = 0;
    // four 32-arc steps at once: the neighbours' priority and degree loads
    // of the four are in flight together
    sweep_light4(
        G, &ws.cursor[0],
        [&](uint32_t v, bool in_range) {
          my[lane] = 0;
          wmy[lane] = 0;
          pv_lane = in_range ? __ldg(&ws.prio[v]) : 0.f;
          rv_lane = in_range ? __ldg(&G.row[v]) : 0u;
          // a degree-1 vertex never looks at its neighbour (but its
          // neighbour may wait for it)
          looks_lane = in_range && __ldg(&G.row[v + 1]) - rv_lane != 1;
          return in_range;
        },
        [&](const bool* valid, const int* owner, const uint32_t* arc) {
          uint32_t u[4], du[4];
          float pu[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            u[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
            arcs += valid[j];
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            pu[j] = valid[j] ? __ldg(&ws.prio[u[j]]) : 0.f;
            du[j] = valid[j] ? __ldg(&G.row[u[j] + 1]) - __ldg(&G.row[u[j]]) : 0u;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float pv = __shfl_sync(kFull, pv_lane, owner[j]);
            const bool looks = __shfl_sync(kFull, looks_lane, owner[j]);
            const uint32_t rv = __shfl_sync(kFull, rv_lane, owner[j]);
            if (valid[j]) {
              if (looks && pu[j] >= pv) atomicAdd(&my[owner[j]], 1u);
              if (pv >= pu[j] && du[j] != 1) ws.wcol[rv + atomicAdd(&wmy[owner[j]], 1u)] = u[j];
            }
          }
        },
        [&](uint32_t v, bool) {
          if (v < G.V && !is_heavy(G, v)) {
            ws.cnt[v] = my[lane];
            ws.wcnt[v] = wmy[lane];
          }
        });
    sweep_heavy(G, &ws.hcursor[0], [&](uint32_t v, uint32_t, uint32_t, uint32_t b, uint32_t e) {
      const float pv = __ldg(&ws.prio[v]);
      const uint32_t rv = __ldg(&G.row[v]);
      uint32_t n = 0;
      // a chunk (kChunk = 128 arcs) as four steps with their loads in flight
      uint32_t u[4], du[4];
      float pu[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t a = b + 32 * j + lane;
        u[j] = a < e ? __ldg(&G.col[a]) : 0u;
        arcs += a < e;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool ok = b + 32 * j + lane < e;
        pu[j] = ok ? __ldg(&ws.prio[u[j]]) : 0.f;
        du[j] = ok ? __ldg(&G.row[u[j] + 1]) - __ldg(&G.row[u[j]]) : 0u;
      }
      unsigned wm[4];
      uint32_t nw = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool ok = b + 32 * j + lane < e;
        n += ok && pu[j] >= pv;
        wm[j] = __ballot_sync(kFull, ok && pv >= pu[j] && du[j] != 1);
        nw += __popc(wm[j]);
      }
      n = warp_add_u32(n);
      if (lane == 0 && n) atomicAdd(&ws.cnt[v], n);
      // the chunk's waiting neighbours: one reservation in v's packed run
      uint32_t at = 0;
      if (lane == 0 && nw) at = atomicAdd(&ws.wcnt[v], nw);
      at = rv + __shfl_sync(kFull, at, 0);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if ((wm[j] >> lane) & 1u) ws.wcol[at + __popc(wm[j] & lanemask_lt())] = u[j];
        at += __popc(wm[j]);
      }
    });
  }
}

// Superstep 2: vertices that wait for nobody take colour 1 (queue slot 1).
__device__ __forceinline__ void color_first(const GraphView& G, const Warps& W, const ColorWs& ws, bool leader,
                                            uint2 (*rstage)[64], unsigned long long& coloured) {
  const int lane = lane_id();
  {
    RangeStage qs{rstage[threadIdx.x >> 5], pick(ws.q, 1), &ws.qcount[1], ws.qcap, ws.overflow};
    for (uint32_t g = W.gwarp; g * 32 < G.V; g += W.nwarps) {
      const uint32_t v = g * 32 + lane;
      const bool first = v < G.V && ld_cg(&ws.cnt[v]) == 0;
      uint32_t rb = 0, wn = 0;
      if (first) {
        ws.color[v] = 1;
        ++coloured;
        rb = __ldg(&G.row[v]);
        wn = ld_cg(&ws.wcnt[v]);
      }
      push_ranges(ws, qs, pick(ws.hc, 1), &ws.hcount[1], first, wn > kHeavyDeg, v, rb, rb + wn);
    }
    qs.flush();
    if (leader) ws.cursor[2] = ws.hcursor[2] = 0;
  }
}

// Round r: the vertices coloured in round r (queue slot r % 3) count down
// the neighbours waiting for them; false when the round has no entries.
__device__ __forceinline__ bool color_round(const GraphView& G, const Warps& W, const ColorWs& ws, uint32_t r,
                                            bool leader, uint2 (*rstage)[64], unsigned long long& arcs,
                                            unsigned long long& coloured) {
  const int lane = lane_id();
  const int cur = r % 3, nxt = (r + 1) % 3, old = (r + 2) % 3;
  // Light groups go to the warps in spread order (warp 0 of every CTA,
  // then warp 1, ...: a small round covers every SM) and heavy chunks to
  // the same order from its other end, so the two lists meet only when a
  // round has more entries than the grid has warps.  In a small round
  // (fewer light entries than two per warp) a warp's light entry is
  // item `ls` and its heavy chunk item `hs`: both loads are issued before
  // the round's counts are known, so they overlap the counts' round trip
  // (entries past the counts are never used).
  const uint32_t ls = W.spread, hs = W.nwarps - 1 - W.spread;
  const uint2* q = pick(ws.q, r);
  const uint4* hc = pick(ws.hc, r);
  uint2 spec = make_uint2(0u, 0u);
  if (lane == 0 && ls < ws.qcap) spec = __ldcg(&q[ls]);
  const uint4 hspec = hs < ws.hcap ? ld_cg(&hc[hs]) : make_uint4(0u, 0u, 0u, 0u);
  const unsigned long long* sc = cta_words<2>([&](unsigned long long* w) {
    w[0] = ld_cg(&ws.qcount[cur]);
    w[1] = __ldcg(&ws.hcount[cur]);
  });
  const uint32_t n = (uint32_t)sc[0];
  const unsigned long long hp = sc[1];
  if (n == 0 && hp == 0) return false;
  if (leader) {
    ws.qcount[old] = 0;
    ws.hcount[old] = 0;
    ws.cursor[old] = 0;
    ws.hcursor[old] = 0;
  }
  RangeStage qs{rstage[threadIdx.x >> 5], pick(ws.q, r + 1), &ws.qcount[nxt], ws.qcap,
                ws.overflow};
  uint4* hc_out = pick(ws.hc, r + 1);
  unsigned long long* hcount_out = &ws.hcount[nxt];
  const int32_t next_color = (int32_t)r + 1;
  // up to four 32-arc steps at once: their neighbour loads and
  // count-downs are all in flight together (a round is a chain of
  // dependent round trips, and thousands of rounds run one after another).
  // Every packed arc leads to a neighbour waiting for this vertex.
  auto relax4 = [&](const bool* valid, const int*, const uint32_t* arc) {
    uint32_t u[4];
#pragma unroll
    for (int s4 = 0; s4 < 4; ++s4) {
      u[s4] = valid[s4] ? __ldcg(&ws.wcol[arc[s4]]) : 0u;
      arcs += valid[s4];
    }
    uint32_t old4[4], rb[4], wn[4];
#pragma unroll
    for (int s4 = 0; s4 < 4; ++s4) {
      old4[s4] = valid[s4] ? atomicSub(&ws.cnt[u[s4]], 1u) : 0u;
      // the packed run of a vertex this count-down may complete, loaded
      // with it
      rb[s4] = valid[s4] ? __ldg(&G.row[u[s4]]) : 0u;
      wn[s4] = valid[s4] ? ld_cg(&ws.wcnt[u[s4]]) : 0u;
    }
#pragma unroll
    for (int s4 = 0; s4 < 4; ++s4) {
      const bool ready = valid[s4] && old4[s4] == 1u;
      if (ready) {
        ws.color[u[s4]] = next_color;
        ++coloured;
      }
      push_ranges(ws, qs, hc_out, hcount_out, ready, wn[s4] > kHeavyDeg, u[s4], rb[s4], rb[s4] + wn[s4]);
    }
  };
  const uint32_t k = group_width(n, W.nwarps);
  WorkTaker lt((n + k - 1) / k, W.nwarps, ls, &ws.cursor[cur]);
  bool first = k == 1;  // the first item taken is the warp's own, ls
  for (uint32_t g = lt.take(); g < lt.n; g = lt.take()) {
    const uint32_t i = g * k + lane;
    const bool act = (uint32_t)lane < k && i < n;
    uint2 rg = make_uint2(0u, 0u);
    if (act) rg = first ? spec : __ldcg(&q[i]);
    first = false;
    range_arcs4(rg.x, rg.y - rg.x, relax4);
  }
  const uint32_t nch = (uint32_t)hp;
  WorkTaker ht(nch, W.nwarps, hs, &ws.hcursor[cur]);
  first = true;  // the first chunk taken is the warp's own, hs
  for (uint32_t c = ht.take(); c < nch; c = ht.take()) {
    const uint4 ent = first ? hspec : ld_cg(&hc[c]);
    first = false;
    const uint32_t b = ent.y, en = ent.z;  // the entry's arc range
    // a chunk holds kChunk = 128 arcs: one four-step batch
    static_assert(kChunk == 4 * 32, "a colour chunk is one batch of four steps");
    bool valid[4];
    uint32_t arc[4];
#pragma unroll
    for (int s4 = 0; s4 < 4; ++s4) {
      arc[s4] = b + 32 * s4 + lane;
      valid[s4] = arc[s4] < en;
    }
    relax4(valid, nullptr, arc);
  }
  qs.flush();
  return true;
}

template <class Sync>
__device__ __forceinline__ void color_body(Sync& s, const GraphView& G, const ColorWs& ws, uint32_t* smem) {
  const Warps W = warps_of(s.id(), s.P());
  const bool leader = s.id() == 0 && threadIdx.x == 0;
  uint32_t* my = smem + (threadIdx.x & ~31u);  // smem: 2 x 512 words
  __shared__ uint2 rstage[kMaxGraphWarps][64];  // per-warp queue staging
  unsigned long long arcs = 0, coloured = 0;
  color_init(G, W, ws);
  if (!s.sync()) return;
  color_count(G, ws, my, my + 512, arcs);
  if (!s.sync()) return;
  color_first(G, W, ws, leader, rstage, coloured);
  if (!s.sync()) return;
  // -- rounds: the vertices coloured in round r (queue slot r % 3) count
  // down the neighbours waiting for them
  uint32_t r = 1;
  for (;; ++r) {
    if (!color_round(G, W, ws, r, leader, rstage, arcs, coloured)) break;
    if (!s.sync()) return;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    arcs += __shfl_xor_sync(kFull, arcs, o);
    coloured += __shfl_xor_sync(kFull, coloured, o);
  }
  if (lane_id() == 0 && arcs) atomicAdd(&ws.stats[0], arcs);
  if (lane_id() == 0 && coloured) atomicAdd(&ws.stats[2], coloured);
  if (leader) ws.stats[1] = r - 1;
}

// One CTA per SM (the rounds are latency-bound; see color_run), so the
// bound leaves the compiler all the registers it wants for the four-step
// batches (R-MAT-22: 33.7 ms at a three-per-SM bound, 31.3 ms).
__global__ void __launch_bounds__(512, 1) k_color_xf(DiscoveryArgs a, GraphView G, ColorWs ws) {
  __shared__ LocalCtx l;
  __shared__ uint32_t smem[1024];
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  color_body(s, G, ws, smem);
}

// Relaunch form (color.cpp:294-334: one launch per superstep, the stop
// flag read back after each): control state s[0] = superstep kind (0:
// count pass, 1: colour 1, 2: round s[1]).
__global__ void k_color_rl_init(GraphView G, ColorWs ws) {
  color_init(G, warps_of(blockIdx.x, gridDim.x), ws);
}

__global__ void __launch_bounds__(512, 1) k_color_rl_step(GraphView G, ColorWs ws, StepCtl* ctl,
                                                         cudaGraphConditionalHandle cond) {
  __shared__ uint32_t smem[1024];
  __shared__ uint2 rstage[kMaxGraphWarps][64];
  const StepCtl& st0 = step_state(ctl);
  const uint32_t kind = st0.s[0], r = st0.s[1];
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long arcs = 0, coloured = 0;
  if (kind == 0)
    color_count(G, ws, smem + (threadIdx.x & ~31u), smem + 512 + (threadIdx.x & ~31u), arcs);
  else if (kind == 1)
    color_first(G, W, ws, leader, rstage, coloured);
  else
    color_round(G, W, ws, r, leader, rstage, arcs, coloured);
  arcs = warp_add_u64(arcs);
  coloured = warp_add_u64(coloured);
  if (lane_id() == 0 && arcs) atomicAdd(&ws.stats[0], arcs);
  if (lane_id() == 0 && coloured) atomicAdd(&ws.stats[2], coloured);
  step_end(ctl, cond, [&](StepCtl& st) {
    if (kind == 0) {
      st.s[0] = 1;
      return true;
    }
    // the next round's entries (slot r + 1), filled by this superstep
    const uint32_t nr = kind == 1 ? 1u : r + 1;
    const int nx = nr % 3;
    const bool more = __ldcg(&ws.qcount[nx]) != 0 || __ldcg(&ws.hcount[nx]) != 0;
    st.s[0] = 2;
    st.s[1] = nr;
    if (!more) ws.stats[1] = nr - 1;
    return more;
  });
}

}  // namespace

using namespace gdbi;

// default_ctas > 0: the launch's CTA count when options.max_ctas and
// options.oversubscribe leave it open.
template <class K, class Ws>
static int launch_xf(gdb_ctx* c, K kernel, const GraphView& G, const Ws& ws, unsigned long long* d_stats,
                     int default_ctas = 0) {
  if (c->opt.barrier != GDB_BARRIER_XF && c->opt.barrier != GDB_BARRIER_XF_FIXED)
    return set_error(c, GDB_ERR_UNSUPPORTED, "this kernel runs on the XF barrier");
  const int block = c->opt.block_size;
  Shape s;
  int rc = persistent_shape(c, (const void*)kernel, block, 0, &s, c->opt.barrier == GDB_BARRIER_XF);
  if (rc) return rc;
  if (default_ctas > 0 && c->opt.max_ctas == 0 && c->opt.oversubscribe == 0)
    s.grid = std::min(s.grid, default_ctas);
  DiscoveryArgs a = discovery_args(c, s);
  c->last = gdb_run_stats{};
  GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  kernel<<<s.grid, block, 0, c->stream>>>(a, G, ws);
  GDB_CUDA(c, cudaGetLastError());
  GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  rc = finish_run(c);
  if (rc) return rc;
  unsigned long long* hs = (unsigned long long*)pinned(c, 64);
  if (!hs) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hs, d_stats, 16, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
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
  return GDB_OK;
}

// Relaunch forms: init once, then one step launch per superstep until the
// step kernels stop (at most `cap` launches); d_stats as for launch_xf.
template <class KI, class KS, class Ws>
static int launch_steps(gdb_ctx* c, KI init, KS step, const GraphView& G, const Ws& ws,
                        unsigned long long* d_stats, StepCtl* ctl, const StepCtl& first,
                        unsigned long long cap, int default_ctas = 0) {
  const int block = c->opt.block_size;
  int grid = 0;
  int rc = step_grid(c, (const void*)step, block, &grid);
  if (rc) return rc;
  if (default_ctas > 0 && c->opt.max_ctas == 0) grid = std::min(grid, default_ctas);
  c->last = gdb_run_stats{};
  rc = step_run(c, c->opt.barrier, (const void*)init, (const void*)step, grid, block, ctl, first, cap,
                true, G, ws);
  if (rc) return rc;
  unsigned long long* hs = (unsigned long long*)pinned(c, 64);
  if (!hs) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hs, d_stats, 16, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  c->last.edges_processed = hs[0];
  c->last.supersteps = (uint32_t)hs[1];
  return GDB_OK;
}

static bool relaunch_kind(const gdb_ctx* c) {
  return c->opt.barrier == GDB_BARRIER_RELAUNCH || c->opt.barrier == GDB_BARRIER_RELAUNCH_GRAPH;
}

static int mis_run(gdb_ctx* c, gdb_graph* g, const float* d_prio, int32_t* d_s) {
  if (!graph_ok(c, g) || !d_prio || !d_s) return GDB_ERR_INVALID;
  const uint32_t hcap = std::max<uint32_t>(g->nheavy, 1);
  Bump b;
  const size_t o_state = b.take((size_t)g->V * 4), o_mn = b.take((size_t)g->V * 4);
  const size_t o_ukey = b.take((size_t)g->V * 4);
  const size_t o_h0 = b.take(hcap * 4), o_h1 = b.take(hcap * 4), o_cnt = b.take(256);
  const size_t o_ctl = b.take(sizeof(StepCtl));
  char* base = (char*)workspace(c, b.off);
  if (!base) return GDB_ERR_OOM;
  MisWs ws;
  ws.state = (int32_t*)(base + o_state);
  ws.ukey = (uint32_t*)(base + o_ukey);
  ws.s = d_s;
  ws.mn = (uint32_t*)(base + o_mn);
  ws.hmn[0] = (uint32_t*)(base + o_h0);
  ws.hmn[1] = (uint32_t*)(base + o_h1);
  ws.prio = d_prio;
  char* cnt = base + o_cnt;
  ws.stats = (unsigned long long*)cnt;
  ws.cursor = (uint32_t*)(cnt + 64);
  ws.hcursor = (uint32_t*)(cnt + 80);
  ws.flag = (uint32_t*)(cnt + 96);
  ws.won = (uint32_t*)(cnt + 112);
  ws.stuck = (int*)(cnt + 128);
  // a round that chooses a vertex decides at least that one: at most V
  // rounds of two phases (a round that chooses none stops the run)
  int rc;
  if (relaunch_kind(c)) {
    StepCtl first{};
    first.s[2] = 1;  // round 0 starts with mis1
    rc = launch_steps(c, k_mis_rl_init, k_mis_rl_step, g->view(), ws, ws.stats, (StepCtl*)(base + o_ctl),
                      first, 2ull * g->V + 4);
  } else {
    rc = launch_xf(c, k_mis_xf, g->view(), ws, ws.stats);
  }
  if (rc) return rc;
  int stuck = 0;
  GDB_CUDA(c, cudaMemcpyAsync(&stuck, ws.stuck, sizeof stuck, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (stuck)
    return set_error(c, GDB_ERR_INVALID,
                     "MIS: a round chose no vertex (adjacent vertices of equal priority, or a NaN "
                     "priority or one of 99999999 and above, never win; the reference never "
                     "terminates then)");
  return GDB_OK;
}

static int color_run(gdb_ctx* c, gdb_graph* g, const float* d_prio, int32_t* d_color) {
  if (!graph_ok(c, g) || !d_prio || !d_color) return GDB_ERR_INVALID;
  const uint32_t V = g->V;
  const uint32_t hcap = chunk_capacity(g);
  Bump b;
  const size_t o_cnt_v = b.take((size_t)V * 4);
  const size_t o_q0 = b.take((size_t)V * 8), o_q1 = b.take((size_t)V * 8);
  const size_t o_hc0 = b.take((size_t)hcap * 16), o_hc1 = b.take((size_t)hcap * 16);
  const size_t o_wcol = b.take(std::max<uint64_t>(g->E, 1) * 4);
  const size_t o_wcnt = b.take((size_t)V * 4);
  const size_t o_cnt = b.take(512);
  const size_t o_ctl = b.take(sizeof(StepCtl));
  char* base = (char*)workspace(c, b.off);
  if (!base) return GDB_ERR_OOM;
  ColorWs ws;
  ws.color = d_color;
  ws.cnt = (uint32_t*)(base + o_cnt_v);
  ws.wcol = (uint32_t*)(base + o_wcol);
  ws.wcnt = (uint32_t*)(base + o_wcnt);
  ws.prio = d_prio;
  ws.q[0] = (uint2*)(base + o_q0);
  ws.q[1] = (uint2*)(base + o_q1);
  ws.hc[0] = (uint4*)(base + o_hc0);
  ws.hc[1] = (uint4*)(base + o_hc1);
  char* cnt = base + o_cnt;
  ws.stats = (unsigned long long*)cnt;             // 4 x u64
  ws.hcount = (unsigned long long*)(cnt + 64);     // 3 x u64
  ws.qcount = (uint32_t*)(cnt + 96);
  ws.cursor = (uint32_t*)(cnt + 112);
  ws.hcursor = (uint32_t*)(cnt + 128);
  ws.overflow = (int*)(cnt + 160);
  ws.qcap = V;
  ws.hcap = hcap;
  GDB_CUDA(c, cudaMemsetAsync(cnt, 0, 512, c->stream));
  // after the count pass a round touches only the arcs of the vertices it
  // colours (thousands of small rounds on power-law graphs): latency-bound,
  // and faster on one CTA per SM (R-MAT-22: 42.8 ms against 47.4 ms on all
  // 456 co-resident CTAs)
  // relaunched: the count pass, colour 1 and at most V rounds
  int rc = relaunch_kind(c) ? launch_steps(c, k_color_rl_init, k_color_rl_step, g->view(), ws, ws.stats,
                                           (StepCtl*)(base + o_ctl), StepCtl{}, (unsigned long long)V + 4,
                                           c->sm_count)
                            : launch_xf(c, k_color_xf, g->view(), ws, ws.stats, c->sm_count);
  if (rc) return rc;
  unsigned long long* h = (unsigned long long*)pinned(c, 4096);
  GDB_CUDA(c, cudaMemcpy(h, cnt, 192, cudaMemcpyDeviceToHost));
  if (*(int*)((char*)h + 160)) return set_error(c, GDB_ERR_CAPACITY, "colour queue overflow");
  if (h[2] != V)
    return set_error(c, GDB_ERR_INVALID,
                     "adjacent vertices of equal priority never take a colour (the reference "
                     "kernel does not terminate on such input)");
  return GDB_OK;
}

// Host-buffer wrapper: copy the priorities in, run, copy the answer out.
template <class Run>
static int with_host_prio(gdb_ctx* c, gdb_graph* g, const float* prio, int32_t* out, Run run) {
  if (!graph_ok(c, g) || !prio || !out) return GDB_ERR_INVALID;
  const size_t n = (size_t)g->V * 4;
  char* d = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, 2 * n, c->stream));
  cudaError_t e = cudaMemcpyAsync(d, prio, n, cudaMemcpyHostToDevice, c->stream);
  int rc = e == cudaSuccess ? run((const float*)d, (int32_t*)(d + n)) : set_cuda_error(c, e, "priorities upload");
  if (rc == GDB_OK) {
    e = cudaMemcpyAsync(out, d + n, n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "result read-back");
  }
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

extern "C" {

int gdb_mis_device(gdb_ctx* c, gdb_graph* g, const float* d_prio, int32_t* d_s) {
  return mis_run(c, g, d_prio, d_s);
}

int gdb_mis(gdb_ctx* c, gdb_graph* g, const float* prio, int32_t* s) {
  return with_host_prio(c, g, prio, s, [&](const float* dp, int32_t* ds) { return mis_run(c, g, dp, ds); });
}

int gdb_color_device(gdb_ctx* c, gdb_graph* g, const float* d_prio, int32_t* d_color) {
  return color_run(c, g, d_prio, d_color);
}

int gdb_color(gdb_ctx* c, gdb_graph* g, const float* prio, int32_t* color) {
  return with_host_prio(c, g, prio, color,
                        [&](const float* dp, int32_t* dc) { return color_run(c, g, dp, dc); });
}

}  // extern "C"
