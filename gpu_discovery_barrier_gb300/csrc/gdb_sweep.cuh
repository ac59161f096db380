// Device building blocks shared by the persistent graph kernels.
//
// Work distribution over a CSR in HBM:
//  * light vertices (degree <= kHeavyDeg) are taken up to 32 at a time by one warp;
//    the warp scans their degrees and walks their concatenated arc lists 32
//    arcs per step, each lane finding the vertex that owns its arc with a
//    5-step shuffle binary search -- consecutive lanes read consecutive
//    column ids, so col[] streams in full 128-byte lines;
//  * heavy vertices (degree > kHeavyDeg) are cut into chunks of kChunk arcs;
//    every chunk is its own work entry {vertex, chunk, vertex slot, chunks},
//    handed out one per warp, so neither a hub nor a sparse superstep's
//    lone medium-degree vertex serialises a superstep;
//  * frontier pushes are warp-aggregated: one atomicAdd per warp and queue.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gdb_discovery.cuh"

namespace gdb {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kHeavyDeg = 128;
constexpr uint32_t kChunk = 128;
// light vertices a warp takes at once (measured on R-MAT-22: 32 beats 8 --
// per-group overhead outweighs the shorter superstep tail)
constexpr uint32_t kGroupMax = 32;
constexpr uint32_t kInf = GDB_LONESTAR_INF;
// groups of 32 vertices a warp takes per atomic on a work cursor (one
// cursor word is shared by every warp of the grid, so grabs are batched)
constexpr uint32_t kGrab = 4;
// warps per CTA of the graph kernels (launch bounds of 512 threads)
constexpr int kMaxGraphWarps = 16;

struct GraphView {
  uint32_t V;
  uint32_t E;
  const uint32_t* __restrict__ row;
  const uint32_t* __restrict__ col;
  const uint32_t* __restrict__ w;
  uint32_t nheavy;
  uint32_t nheavy_chunks;
  const uint32_t* __restrict__ heavy_v;     // ascending ids
  const uint4* __restrict__ heavy_chunk;    // {vertex, chunk, heavy index, chunks}
  const uint32_t* __restrict__ heavy_bits;  // membership bitmap
};

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
__device__ __forceinline__ bool is_heavy(const GraphView& G, uint32_t v) {
  return (__ldg(&G.heavy_bits[v >> 5]) >> (v & 31)) & 1u;
}
__host__ __device__ __forceinline__ uint32_t chunks_of(uint32_t deg) { return (deg + kChunk - 1) / kChunk; }

// Loads that bypass L1 for arrays other CTAs update during the kernel.
__device__ __forceinline__ uint32_t ld_cg(const uint32_t* p) { return __ldcg(p); }
__device__ __forceinline__ int32_t ld_cg(const int32_t* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_cg(const float* p) { return __ldcg(p); }
__device__ __forceinline__ unsigned long long ld_cg(const unsigned long long* p) { return __ldcg(p); }
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ uint4 ld_cg(const uint4* p) { return __ldcg(p); }

// a[i & 1] without dynamic indexing (which would copy the kernel-parameter
// array to local memory).
template <class T>
__device__ __forceinline__ T pick(const T (&a)[2], uint32_t i) {
  return (i & 1) ? a[1] : a[0];
}

// Order-preserving float <-> uint32 map (so atomicMin/Max on uint32 order
// floats; -0 is folded onto +0 first).
__device__ __forceinline__ uint32_t fkey(float f) {
  uint32_t b = __float_as_uint(f == 0.0f ? 0.0f : f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
  uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(b);
}

// Warp identity among the participating CTAs.
struct Warps {
  uint32_t gwarp;   // global warp index
  uint32_t nwarps;  // warps in the participating grid
  uint32_t gthread;
  uint32_t nthreads;
  uint32_t spread;  // warp index counted across the CTAs first (warp 0 of every CTA, then warp 1, ...)
};
__device__ __forceinline__ Warps warps_of(int id, int P) {
  Warps w;
  const uint32_t wpb = blockDim.x >> 5;
  w.gwarp = (uint32_t)id * wpb + (threadIdx.x >> 5);
  w.spread = (threadIdx.x >> 5) * (uint32_t)P + (uint32_t)id;
  w.nwarps = (uint32_t)P * wpb;
  w.gthread = (uint32_t)id * blockDim.x + threadIdx.x;
  w.nthreads = (uint32_t)P * blockDim.x;
  return w;
}

// Lane 0 takes the next ticket from a global cursor; broadcast to the warp.
__device__ __forceinline__ uint32_t warp_grab(uint32_t* cursor) {
  uint32_t t = 0;
  if (lane_id() == 0) t = atomicAdd(cursor, 1u);
  return __shfl_sync(kFull, t, 0);
}

// Work items [0, n) over the warps of the grid: each warp first takes one
// item without any atomic, then -- only when there are more items than
// warps -- keeps taking tickets nwarps + cursor++.  Small frontiers
// (thousands of rounds of colouring, the tail levels of traversals) cost no
// atomics.  `after` rotates the assignment so that a second list (heavy
// chunks after light groups) starts on the warps the first left idle
// instead of queueing behind it on the same warps.  The first items go to
// the warps of CTA 0 first (the SSSP supersteps: 21.1 ms against 21.9 with
// the spread order).
struct WorkTaker {
  uint32_t n, nwarps, next;
  uint32_t* cursor;
  __device__ __forceinline__ WorkTaker(uint32_t n_, const Warps& W, uint32_t* c, uint32_t after = 0)
      : n(n_), nwarps(W.nwarps), cursor(c) {
    const uint32_t off = after % nwarps;
    next = W.gwarp >= off ? W.gwarp - off : W.gwarp + nwarps - off;
  }
  // slot: this warp's own item, any one-to-one map of the grid's warps
  // onto [0, nwarps)
  __device__ __forceinline__ WorkTaker(uint32_t n_, uint32_t nwarps_, uint32_t slot, uint32_t* c)
      : n(n_), nwarps(nwarps_), next(slot), cursor(c) {}
  // next item or n when done
  __device__ __forceinline__ uint32_t take() {
    const uint32_t g = next;
    if (g >= n) return n;
    next = n <= nwarps ? n : nwarps + warp_grab(cursor);
    return g;
  }
};

// Walk the arcs of the (active, light) vertices held by the 32 lanes.
// Calls fn(valid, owner_lane, arc) once per 32-arc step with every lane
// present, so fn may use warp collectives; `valid` marks lanes with an arc.
template <class Fn>
__device__ __forceinline__ void group_arcs(const GraphView& G, bool active, uint32_t v, Fn&& fn) {
  const int lane = lane_id();
  uint32_t beg = 0, deg = 0;
  if (active) {
    beg = __ldg(&G.row[v]);
    deg = __ldg(&G.row[v + 1]) - beg;
  }
  uint32_t pre = deg;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(kFull, pre, o);
    if (lane >= o) pre += t;
  }
  const uint32_t total = __shfl_sync(kFull, pre, 31);
  pre -= deg;
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t k = base + lane;
    int lo = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      uint32_t p = __shfl_sync(kFull, pre, lo + s);
      if (p <= k) lo += s;
    }
    const uint32_t obeg = __shfl_sync(kFull, beg, lo);
    const uint32_t opre = __shfl_sync(kFull, pre, lo);
    fn(k < total, lo, obeg + (k - opre));
  }
}

// group_arcs four steps at a time: fn(valid[4], owner[4], arc[4]) receives
// the arcs (and owner lanes) of up to four consecutive 32-arc steps, so
// that the caller can issue their loads and atomics together -- one round
// trip per four steps on latency-bound paths instead of one per step.
// The arcs come as the lanes' ranges [beg, beg + deg) (deg = 0: none).
template <class Fn>
__device__ __forceinline__ void range_arcs4(uint32_t beg, uint32_t deg, Fn&& fn) {
  const int lane = lane_id();
  uint32_t pre = deg;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(kFull, pre, o);
    if (lane >= o) pre += t;
  }
  const uint32_t total = __shfl_sync(kFull, pre, 31);
  pre -= deg;
  for (uint32_t base = 0; base < total; base += 128) {
    bool valid[4] = {false, false, false, false};
    int owner[4] = {0, 0, 0, 0};
    uint32_t arc[4] = {0, 0, 0, 0};
#pragma unroll
    for (int s4 = 0; s4 < 4; ++s4) {
      if (base + 32 * s4 >= total) break;  // warp-uniform: no owner search for empty steps
      const uint32_t k = base + 32 * s4 + lane;
      int lo = 0;
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) {
        uint32_t p = __shfl_sync(kFull, pre, lo + s);
        if (p <= k) lo += s;
      }
      const uint32_t obeg = __shfl_sync(kFull, beg, lo);
      const uint32_t opre = __shfl_sync(kFull, pre, lo);
      valid[s4] = k < total;
      owner[s4] = lo;
      arc[s4] = obeg + (k - opre);
    }
    fn(valid, owner, arc);
  }
}

template <class Fn>
__device__ __forceinline__ void group_arcs4(const GraphView& G, bool active, uint32_t v, Fn&& fn) {
  uint32_t beg = 0, deg = 0;
  if (active) {
    beg = __ldg(&G.row[v]);
    deg = __ldg(&G.row[v + 1]) - beg;
  }
  range_arcs4(beg, deg, fn);
}

// Walk arcs [b, e) of one vertex, 32 per step, every lane present.
template <class Fn>
__device__ __forceinline__ void range_arcs(uint32_t b, uint32_t e, Fn&& fn) {
  const int lane = lane_id();
  for (uint32_t a0 = b; a0 < e; a0 += 32) {
    const uint32_t a = a0 + lane;
    fn(a < e, a);
  }
}

// Vertices per warp group for a frontier of n light vertices: kGroupMax
// when there is enough work for every warp, fewer (down to one vertex per
// warp) when the frontier is small, so sparse supersteps spread over all
// warps.
__device__ __forceinline__ uint32_t group_width(uint32_t n, uint32_t nwarps) {
  if (n >= kGroupMax * nwarps) return kGroupMax;
  const uint32_t k = n / nwarps;
  return k < 1u ? 1u : k;
}

// A frontier: a queue of light vertices plus one work entry per heavy chunk,
// {vertex, chunk index, vertex slot, chunks of the vertex}.  One packed
// 64-bit atomicAdd on hcount reserves a vertex slot (high word) and the
// vertex's run of chunk entries (low word).
struct Frontier {
  uint32_t* q;        // light vertices
  uint4* hc;          // heavy chunk entries
  uint32_t* qcount;   // light count
  unsigned long long* hcount;  // (vertex slots << 32) | chunk entries
  uint32_t qcap, hcap;         // capacities: light vertices, chunk entries
  int* overflow;      // set when a push would exceed a capacity
  uint32_t vcap = 0xffffffffu;  // optional: vertex-slot capacity
  uint32_t* hleft = nullptr;    // optional: chunk countdown per slot, armed at push
  double* hacc = nullptr;       // optional: FP64 accumulator per slot, cleared at push
};

// The lanes' `heavy` vertices: their degrees are loaded together, one
// packed atomic on the frontier's heavy counter reserves every vertex slot
// and chunk entry of the warp's heavy vertices at once, and the warp then
// writes each vertex's entries together -- no round trip per vertex (a
// level whose arcs claim thousands of hubs otherwise serialises on them).
__device__ __forceinline__ void frontier_push_heavy(const GraphView& G, const Frontier& F,
                                                    bool heavy, uint32_t v) {
  const unsigned hm = __ballot_sync(kFull, heavy);
  if (!hm) return;
  const int lane = lane_id();
  const uint32_t nch = heavy ? chunks_of(__ldg(&G.row[v + 1]) - __ldg(&G.row[v])) : 0u;
  uint32_t inc = nch;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  const uint32_t total = __shfl_sync(kFull, inc, 31);
  const uint32_t cofs = inc - nch;  // this lane's first entry, relative
  const uint32_t nh = __popc(hm);
  const int leader = __ffs(hm) - 1;
  unsigned long long old = 0;
  if (lane == leader) old = atomicAdd(F.hcount, ((unsigned long long)nh << 32) | total);
  old = __shfl_sync(kFull, old, leader);
  const uint32_t vslot0 = (uint32_t)(old >> 32), cbase0 = (uint32_t)old;
  if (cbase0 + total > F.hcap || vslot0 + nh > F.vcap) {
    if (lane == leader) atomicExch(F.overflow, 1);
    return;
  }
  if (heavy && F.hleft) {
    const uint32_t vs = vslot0 + __popc(hm & lanemask_lt());
    F.hleft[vs] = nch;
    F.hacc[vs] = -0.0;  // an empty sum (segment_add)
  }
  for (unsigned m = hm; m; m &= m - 1) {
    const int l = __ffs(m) - 1;
    const uint32_t hvx = __shfl_sync(kFull, v, l), n = __shfl_sync(kFull, nch, l);
    const uint32_t cb = cbase0 + __shfl_sync(kFull, cofs, l);
    const uint32_t vs = vslot0 + __popc(hm & ((1u << l) - 1u));
    for (uint32_t j = lane; j < n; j += 32) F.hc[cb + j] = make_uint4(hvx, j, vs, n);
  }
}

// Warp-aggregated push of the lanes' `want` vertices (one atomic per warp
// step on the light counter).
__device__ __forceinline__ void frontier_push(const GraphView& G, const Frontier& F, bool want,
                                              uint32_t v) {
  const int lane = lane_id();
  const bool heavy = want && is_heavy(G, v);
  const bool light = want && !heavy;
  const unsigned m = __ballot_sync(kFull, light);
  if (m) {
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(F.qcount, (uint32_t)__popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (light) {
      const uint32_t slot = base + __popc(m & lanemask_lt());
      if (slot < F.qcap) F.q[slot] = v;
      else atomicExch(F.overflow, 1);
    }
  }
  frontier_push_heavy(G, F, heavy, v);
}

// Per-warp staging of queue appends in shared memory: the lanes' entries
// collect in the warp's 64-slot buffer and leave 32 at a time with one
// counter atomic, instead of one atomic per warp step -- a counter word
// that every warp of the grid hits is an L2 hot spot.  flush() before the
// superstep's barrier.
struct WarpStage {
  uint32_t* buf;     // this warp's 64 slots
  uint32_t* q;       // the queue and its counter
  uint32_t* count;
  uint32_t cap;
  int* overflow;
  uint32_t n = 0;    // staged entries (warp-uniform)

  __device__ __forceinline__ void out(uint32_t x, uint32_t m) {
    const int lane = lane_id();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(count, m);
    base = __shfl_sync(kFull, base, 0);
    if ((uint32_t)lane < m) {
      if (base + lane < cap) q[base + lane] = x;
      else atomicExch(overflow, 1);
    }
  }
  __device__ __forceinline__ void add(bool want, uint32_t v) {
    const unsigned m = __ballot_sync(kFull, want);
    if (!m) return;
    const int lane = lane_id();
    if (want) buf[n + __popc(m & lanemask_lt())] = v;
    n += __popc(m);
    if (n >= 32) {
      __syncwarp();
      const uint32_t x = buf[lane], r = n - 32;
      const uint32_t y = (uint32_t)lane < r ? buf[32 + lane] : 0u;
      __syncwarp();
      if ((uint32_t)lane < r) buf[lane] = y;
      __syncwarp();
      out(x, 32);
      n = r;
    }
  }
  __device__ __forceinline__ void flush() {
    __syncwarp();
    if (n) out((uint32_t)lane_id() < n ? buf[lane_id()] : 0u, n);
    n = 0;
  }
};

// This warp's 64-slot staging buffer number k (0-2), shared by the
// staged queues of a superstep.
__device__ __forceinline__ uint32_t* warp_stage(int k) {
  __shared__ uint32_t buf[3][kMaxGraphWarps][64];
  return buf[k][threadIdx.x >> 5];
}

// A staged frontier: light entries through the warp's buffer k.
__device__ __forceinline__ WarpStage frontier_stage(const Frontier& F, int k) {
  return WarpStage{warp_stage(k), F.q, F.qcount, F.qcap, F.overflow};
}

// frontier_push with the light entries staged.
__device__ __forceinline__ void frontier_push_staged(const GraphView& G, const Frontier& F,
                                                     WarpStage& st, bool want, uint32_t v) {
  const bool heavy = want && is_heavy(G, v);
  st.add(want && !heavy, v);
  frontier_push_heavy(G, F, heavy, v);
}

// One thread seeds a frontier with vertex v (the traversal's source).
__device__ __forceinline__ void frontier_seed(const GraphView& G, const Frontier& F, uint32_t v) {
  if (is_heavy(G, v)) {
    const uint32_t nch = chunks_of(G.row[v + 1] - G.row[v]);
    for (uint32_t j = 0; j < nch; ++j) F.hc[j] = make_uint4(v, j, 0u, nch);
    if (F.hleft) {
      F.hleft[0] = nch;
      F.hacc[0] = -0.0;  // an empty sum (segment_add)
    }
    *F.hcount = (1ull << 32) | nch;
  } else {
    F.q[0] = v;
    *F.qcount = 1;
  }
}

// Many sources at once: the grid's warps push every source not seen before
// (CAS on its distance from `unreached` to 0) into frontier F.  Used for
// batches: on a disjoint union of graphs with one source per graph, each
// vertex is reached only from its own graph's source.
__device__ __forceinline__ void frontier_seed_many(const GraphView& G, const Frontier& F,
                                                   const Warps& W, const uint32_t* srcs,
                                                   uint32_t nsrc, uint32_t* dist,
                                                   uint32_t unreached,
                                                   unsigned long long* arcs_out = nullptr) {
  const int lane = lane_id();
  unsigned long long arcs = 0;
  for (uint32_t base = W.gwarp * 32; base < nsrc; base += W.nwarps * 32) {
    const uint32_t i = base + lane;
    bool want = i < nsrc;
    const uint32_t v = want ? __ldg(&srcs[i]) : 0u;
    if (v >= G.V) want = false;  // out-of-range sources are ignored
    if (want) want = atomicCAS(&dist[v], unreached, 0u) == unreached;
    if (want && arcs_out) arcs += __ldg(&G.row[v + 1]) - __ldg(&G.row[v]);
    frontier_push(G, F, want, v);
  }
  if (arcs_out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) arcs += __shfl_xor_sync(0xffffffffu, arcs, o);
    if (lane == 0 && arcs) atomicAdd(arcs_out, arcs);
  }
}

// Arc range [b, e) of heavy chunk entry `ent`.
__device__ __forceinline__ void chunk_range(const GraphView& G, const uint4& ent, uint32_t& b,
                                            uint32_t& e) {
  const uint32_t rb = __ldg(&G.row[ent.x]), re = __ldg(&G.row[ent.x + 1]);
  b = rb + ent.y * kChunk;
  e = min(re, b + kChunk);
}

// Visit a frontier: light vertices in warp groups of 32, then heavy chunks.
// light(valid, owner_lane, owner_vertex_in_lane, arc) is called through
// group_arcs; heavy(valid, v, arc) per 32-arc step of a chunk.
template <class Light, class Heavy>
__device__ __forceinline__ void visit_frontier(const GraphView& G, const Warps& W, const uint32_t* q,
                                               uint32_t n, const uint4* hc,
                                               unsigned long long hpacked, uint32_t* cursor,
                                               uint32_t* hcursor, Light&& light, Heavy&& heavy) {
  const int lane = lane_id();
  const uint32_t k = group_width(n, W.nwarps);
  WorkTaker lt((n + k - 1) / k, W, cursor);
  for (uint32_t g = lt.take(); g < lt.n; g = lt.take()) {
    const uint32_t i = g * k + lane;
    const bool act = (uint32_t)lane < k && i < n;
    const uint32_t v = act ? ld_cg(&q[i]) : 0u;
    group_arcs(G, act, v, [&](bool valid, int owner, uint32_t arc) { light(valid, owner, v, arc); });
  }
  const uint32_t nch = (uint32_t)hpacked;
  WorkTaker ht(nch, W, hcursor, lt.n);
  for (uint32_t c = ht.take(); c < nch; c = ht.take()) {
    const uint4 ent = ld_cg(&hc[c]);
    uint32_t b, en;
    chunk_range(G, ent, b, en);
    range_arcs(b, en, [&](bool valid, uint32_t arc) { heavy(valid, ent.x, arc); });
  }
}

// visit_frontier with four 32-arc steps per call of edge4(valid[4], arc[4]):
// light groups through group_arcs4, a heavy chunk (kChunk = 128 arcs) as
// its four steps.
template <class Edge4>
__device__ __forceinline__ void visit_frontier4(const GraphView& G, const Warps& W, const uint32_t* q,
                                                uint32_t n, const uint4* hc, unsigned long long hpacked,
                                                uint32_t* cursor, uint32_t* hcursor, Edge4&& edge4) {
  static_assert(kChunk == 4 * 32, "a chunk is four steps");
  const int lane = lane_id();
  const uint32_t k = group_width(n, W.nwarps);
  WorkTaker lt((n + k - 1) / k, W, cursor);
  for (uint32_t g = lt.take(); g < lt.n; g = lt.take()) {
    const uint32_t i = g * k + lane;
    const bool act = (uint32_t)lane < k && i < n;
    const uint32_t v = act ? ld_cg(&q[i]) : 0u;
    group_arcs4(G, act, v, [&](const bool* valid, const int*, const uint32_t* arc) { edge4(valid, arc); });
  }
  const uint32_t nch = (uint32_t)hpacked;
  WorkTaker ht(nch, W, hcursor, lt.n);
  for (uint32_t c = ht.take(); c < nch; c = ht.take()) {
    const uint4 ent = ld_cg(&hc[c]);
    uint32_t b, en;
    chunk_range(G, ent, b, en);
    bool valid[4];
    uint32_t arc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      arc[j] = b + 32 * j + lane;
      valid[j] = arc[j] < en;
    }
    edge4(valid, arc);
  }
}

// Sweep the light vertices of [0, V) in warp groups of 32 consecutive ids.
// begin(v, in_range) -> bool active: per-lane setup (v is light and < V
// when in_range); edge(valid, owner_lane, arc) per 32-arc step;
// end(v, active) after the group's arcs.  Groups come from `cursor`.
template <class Begin, class Edge, class End>
__device__ __forceinline__ void sweep_light(const GraphView& G, uint32_t* cursor, Begin&& begin,
                                            Edge&& edge, End&& end) {
  const int lane = lane_id();
  const uint32_t ngroups = (G.V + 31) / 32;
  for (;;) {
    const uint32_t g0 = warp_grab(cursor) * kGrab;
    if (g0 >= ngroups) break;
    for (uint32_t g = g0; g < min(g0 + kGrab, ngroups); ++g) {
      const uint32_t v = g * 32 + lane;
      const bool in_range = v < G.V && !is_heavy(G, v);
      const bool act = begin(v, in_range) && in_range;
      __syncwarp();
      group_arcs(G, act, v, edge);
      __syncwarp();
      end(v, act);
    }
  }
}

// sweep_light with four 32-arc steps per call of edge4(valid[4],
// owner_lane[4], arc[4]) (group_arcs4), so a step's dependent loads are in
// flight together with the next three steps'.
template <class Begin, class Edge4, class End>
__device__ __forceinline__ void sweep_light4(const GraphView& G, uint32_t* cursor, Begin&& begin,
                                             Edge4&& edge4, End&& end) {
  const int lane = lane_id();
  const uint32_t ngroups = (G.V + 31) / 32;
  for (;;) {
    const uint32_t g0 = warp_grab(cursor) * kGrab;
    if (g0 >= ngroups) break;
    for (uint32_t g = g0; g < min(g0 + kGrab, ngroups); ++g) {
      const uint32_t v = g * 32 + lane;
      const bool in_range = v < G.V && !is_heavy(G, v);
      const bool act = begin(v, in_range) && in_range;
      __syncwarp();
      group_arcs4(G, act, v, edge4);
      __syncwarp();
      end(v, act);
    }
  }
}

// Sweep the heavy vertices through the static chunk table, kGrab chunks
// per grab: fn(chunk, v, heavy_index, chunk_in_vertex, arc_begin, arc_end),
// chunk = the entry's index in the table.
template <class Fn>
__device__ __forceinline__ void sweep_heavy_indexed(const GraphView& G, uint32_t* hcursor, Fn&& fn) {
  for (;;) {
    const uint32_t c0 = warp_grab(hcursor) * kGrab;
    if (c0 >= G.nheavy_chunks) break;
    for (uint32_t c = c0; c < min(c0 + kGrab, G.nheavy_chunks); ++c) {
      const uint4 ent = __ldg(&G.heavy_chunk[c]);
      uint32_t b, en;
      chunk_range(G, ent, b, en);
      fn(c, ent.x, ent.z, ent.y, b, en);
    }
  }
}

// sweep_heavy_indexed without the chunk index:
// fn(v, heavy_index, chunk_in_vertex, arc_begin, arc_end).
template <class Fn>
__device__ __forceinline__ void sweep_heavy(const GraphView& G, uint32_t* hcursor, Fn&& fn) {
  sweep_heavy_indexed(G, hcursor, [&](uint32_t, uint32_t v, uint32_t h, uint32_t j, uint32_t b, uint32_t e) {
    fn(v, h, j, b, e);
  });
}

// Warp reductions.
__device__ __forceinline__ uint32_t warp_min_u32(uint32_t x) { return __reduce_min_sync(kFull, x); }
__device__ __forceinline__ uint32_t warp_max_u32(uint32_t x) { return __reduce_max_sync(kFull, x); }
__device__ __forceinline__ uint32_t warp_or_u32(uint32_t x) { return __reduce_or_sync(kFull, x); }
__device__ __forceinline__ uint32_t warp_add_u32(uint32_t x) { return __reduce_add_sync(kFull, x); }
__device__ __forceinline__ unsigned long long warp_add_u64(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
  return x;
}
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long y = __shfl_xor_sync(kFull, x, o);
    x = y < x ? y : x;
  }
  return x;
}
// Words every thread of the CTA needs at the start of a superstep (queue
// counts, flags, level bounds): thread 0 loads them and the CTA shares
// them through shared memory.  Thousands of warps loading one word at the
// same moment queue on a single L2 slice; on the 4096^2 grid BFS that
// queueing was more than a third of the level time.  Every thread of the
// CTA calls it (two CTA barriers).
// (Load fills N words; the words stay readable until the next call of the
// same instantiation.)
template <int N, class Load>
__device__ __forceinline__ const unsigned long long* cta_words(Load&& load) {
  __shared__ unsigned long long s[N];
  __syncthreads();
  if (threadIdx.x == 0) load(s);
  __syncthreads();
  return s;
}

// Count-down of *p by one with acquire-release semantics: this thread's
// earlier writes are ordered before it, and the thread that takes the
// count to zero sees the writes of every thread that counted down before
// it (a fence-free completion pattern; __threadfence is a full fence).
__device__ __forceinline__ uint32_t countdown_acq_rel(uint32_t* p) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;"
               : "=r"(old)
               : "l"(p), "r"(0xFFFFFFFFu)
               : "memory");
  return old;
}

// One atomicOr of `bit` into *word per CTA when any of its threads has `p`
// (instead of one per warp).  Every thread of the CTA calls it.
__device__ __forceinline__ void cta_or(bool p, uint32_t* word, uint32_t bit) {
  if (__syncthreads_or(p) && threadIdx.x == 0) atomicOr(word, bit);
}

// Per-owner sums of one group_arcs step.  Owners never decrease from lane
// to lane, so each owner's lanes are contiguous: a segmented suffix scan
// leaves every segment's total in its first lane, which adds it to
// slot[owner] -- one lane per owner per step, no atomics.  Every lane of
// the warp calls it.  The scan runs in FP32 and only the segment totals
// are added in FP64 (one FP64 add per owner per step instead of five per
// arc: FP64 issues at a small fraction of the FP32 rate on this GPU).
// -0.0 is the neutral term: a segment of -0.0 leaves its slot untouched, so
// a slot that starts at -0.0 still reads -0.0 when nothing was added.
__device__ __forceinline__ void segment_add(double* slot, int owner, float x) {
  const int lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float y = __shfl_down_sync(kFull, x, o);
    const int ow = __shfl_down_sync(kFull, owner, o);
    if (lane + o < 32 && ow == owner) x += y;
  }
  const int prev = __shfl_up_sync(kFull, owner, 1);
  if ((lane == 0 || prev != owner) && __float_as_uint(x) != 0x80000000u) slot[owner] += (double)x;
}

__device__ __forceinline__ float warp_sum_f32(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
  return x;
}

// Barrier abstraction for the persistent kernels: XF over discovered CTAs
// or cooperative_groups grid sync over a cooperative launch.
// Grid barriers for the persistent bodies.  sync_hook(h): h runs once, in
// CTA 0 (all its threads), between the last arrival and the release.
struct XfSync {
  const DiscoveryArgs* a;
  LocalCtx* l;
  __device__ ~XfSync() { xf_finish(*a, l); }
  __device__ __forceinline__ bool sync() { return xf_barrier(*a, l); }
  template <class H>
  __device__ __forceinline__ bool sync_hook(H&& h) {
    return xf_barrier(*a, l, h);
  }
  __device__ __forceinline__ int id() const { return l->id; }
  __device__ __forceinline__ int P() const { return l->P; }
};
struct GridSync {
  __device__ __forceinline__ bool sync() {
    cooperative_groups::this_grid().sync();
    return true;
  }
  template <class H>
  __device__ __forceinline__ bool sync_hook(H&& h) {
    cooperative_groups::this_grid().sync();
    if (blockIdx.x == 0) h();
    cooperative_groups::this_grid().sync();
    return true;
  }
  __device__ __forceinline__ int id() const { return blockIdx.x; }
  __device__ __forceinline__ int P() const { return gridDim.x; }
};

}  // namespace gdb
