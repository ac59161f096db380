// Minimum spanning forest by Boruvka rounds in one persistent kernel.
//
// Replaces the LonestarGPU MST (host loop lonestar/apps/mst/mst_port.cpp:202-312
// over dinit/dfindelemin/dfindelemin2/verify_min_elem, mst_common.cl:41-194,
// and the persistent dfindcompmintwo, mst_port_kernel.cl:35-82).  The
// reference leaves the device after every kernel and after every `repeat`
// of dfindcompmintwo to read two words; here the whole round loop stays on
// the device behind the XF barrier.  A round:
//   A. every vertex finds its lightest arc to another component and
//      atomicMin's the key (weight << 32 | arc) into its component's slot
//      (dfindelemin + dfindelemin2 in one step: the arc index breaks ties).
//      Components only merge, so the arcs of a unit (a light vertex, or a
//      128-arc chunk of a heavy one) that leave its component only become
//      fewer: while the lightest of them found by the unit's last scan
//      still leaves the component, it is still the lightest, and a unit
//      that found none never finds one.  A heavy chunk also keeps its
//      second lightest such arc, which takes over when the first turns
//      internal.  A unit scans its arcs again only when its kept arcs have
//      turned internal;
//   B1. every component root records the root its lightest arc reaches;
//   B2. roots hook onto that root, except a root whose arc weighs the same
//      as the target root's arc and whose id is the smaller, which stays a
//      root (cs_unify breaks cycles by id too, component_cl.h:58-64); each
//      hook adds its arc's weight once.  With unique weights an equal
//      weight means the same edge, so this is the smaller id of a mutual
//      pair.  With equal weights on different edges, ties between arc
//      indices differ by direction and could close a cycle of hooks;
//      (weight, id) falls strictly along every hook instead, so no cycle
//      forms, and each round still hooks at least one root that has an
//      arc leaving its component;
//   C. pointer jumping flattens every vertex onto its root.
// With unique weights the forest is unique, so weight, edge count and edge
// set equal the reference's.  The weight is kept exactly (uint64) and also
// as the reference's wrapping uint32 sum (mst_port_kernel.cl:69); arcs of
// weight >= 1e9 are never chosen (mst_common.cl:84-88).
#include <algorithm>

#include "gdb_internal.h"

namespace {

using namespace gdb;

constexpr unsigned long long kNoArc = ~0ull;
// A unit's kept arc (vcand per light vertex; hcand.x per heavy chunk, with
// the second lightest in hcand.y): a key, kScan (scan the unit's arcs; for
// hcand.y: not known) or kNone (no arc leaves its component, for good; for
// hcand.y: no second one).  Keys stay below 2^62 (weights below kInf).
constexpr unsigned long long kScan = ~0ull;
constexpr unsigned long long kNone = ~0ull - 1;

struct MstWs {
  uint32_t* comp;
  unsigned long long* best;
  unsigned long long* vcand;     // per vertex (light vertices)
  ulonglong2* hcand;             // per heavy chunk: the two lightest
  uint32_t* partner;
  uint8_t* arc_flag;             // nullable
  uint32_t* cursor;              // [3]
  uint32_t* hcursor;             // [3]
  uint32_t* hooks;               // [3]
  int* stuck;                    // set if pointer jumping ever meets a cycle (see C)
  unsigned long long* acc;       // [0] weight, [1] edges, [2] rounds, [3] arcs inspected
};

template <class Sync>
__device__ __forceinline__ void mst_body(Sync& s, const GraphView& G, const MstWs& ws,
                                         unsigned long long* smem) {
  const Warps W = warps_of(s.id(), s.P());
  const bool leader = s.id() == 0 && threadIdx.x == 0;
  const int lane = lane_id();
  unsigned long long* my = smem + (threadIdx.x & ~31u);
  for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
    ws.comp[v] = v;
    ws.best[v] = kNoArc;
    ws.vcand[v] = kScan;
  }
  for (uint32_t c = W.gthread; c < G.nheavy_chunks; c += W.nthreads) ws.hcand[c] = make_ulonglong2(kScan, kScan);
  if (ws.arc_flag)
    for (uint32_t a = W.gthread; a < G.E; a += W.nthreads) ws.arc_flag[a] = 0;
  if (leader) {
    for (int i = 0; i < 3; ++i) ws.cursor[i] = ws.hcursor[i] = ws.hooks[i] = 0;
    for (int i = 0; i < 4; ++i) ws.acc[i] = 0;
    *ws.stuck = 0;
  }
  if (!s.sync()) return;
  unsigned long long arcs = 0, wsum = 0, nedges = 0;
  uint32_t t = 0, round = 0;
  // a round with a hook merges two components at least: V rounds bound
  // the loop
  for (; round <= G.V; ++round) {
    // ---- A: lightest arc leaving each vertex's component
    {
      const int cur = t % 3, old = (t + 2) % 3;
      if (leader) ws.cursor[old] = ws.hcursor[old] = ws.hooks[old] = 0;
      uint32_t cv = 0;
      // four 32-arc steps at once: their weight, column and component
      // loads are in flight together
      sweep_light4(
          G, &ws.cursor[cur],
          [&](uint32_t v, bool in_range) {
            my[lane] = kNoArc;
            cv = in_range ? ld_cg(&ws.comp[v]) : 0u;
            if (!in_range) return false;
            const unsigned long long k = ld_cg(&ws.vcand[v]);
            if (k == kNone) return false;
            if (k != kScan && ld_cg(&ws.comp[__ldg(&G.col[(uint32_t)k])]) != cv) {
              // the kept arc still leaves the component
              if (k < ld_cg(&ws.best[cv])) atomicMin(&ws.best[cv], k);
              return false;
            }
            return true;
          },
          [&](const bool* valid, const int* owner, const uint32_t* arc) {
            uint32_t wt[4], cu[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              wt[k] = valid[k] ? __ldg(&G.w[arc[k]]) : kInf;
              cu[k] = wt[k] < kInf ? __ldg(&G.col[arc[k]]) : 0u;
              arcs += valid[k];
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) cu[k] = wt[k] < kInf ? ld_cg(&ws.comp[cu[k]]) : 0u;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const uint32_t co = __shfl_sync(kFull, cv, owner[k]);
              if (wt[k] < kInf && cu[k] != co) {
                const unsigned long long key = ((unsigned long long)wt[k] << 32) | arc[k];
                if (key < my[owner[k]]) atomicMin(&my[owner[k]], key);
              }
            }
          },
          [&](uint32_t v, bool act) {
            if (!act) return;
            ws.vcand[v] = my[lane] == kNoArc ? kNone : my[lane];
            if (my[lane] != kNoArc && my[lane] < ld_cg(&ws.best[cv])) atomicMin(&ws.best[cv], my[lane]);
          });
      sweep_heavy_indexed(G, &ws.hcursor[cur], [&](uint32_t ci, uint32_t v, uint32_t, uint32_t, uint32_t b,
                                                    uint32_t e) {
        const uint32_t c = ld_cg(&ws.comp[v]);
        const ulonglong2 kept = __ldcg(&ws.hcand[ci]);
        if (kept.x == kNone) return;
        if (kept.x != kScan) {
          // both kept arcs checked at once
          const bool two = kept.y != kScan && kept.y != kNone;
          const uint32_t u1 = __ldg(&G.col[(uint32_t)kept.x]);
          const uint32_t u2 = two ? __ldg(&G.col[(uint32_t)kept.y]) : 0u;
          const bool out1 = ld_cg(&ws.comp[u1]) != c;
          const bool out2 = two && ld_cg(&ws.comp[u2]) != c;
          unsigned long long use = kNoArc;
          if (out1) {
            use = kept.x;
          } else if (kept.y == kNone) {
            // the only arc that left the chunk's component is internal now
            if (lane == 0) ws.hcand[ci].x = kNone;
            return;
          } else if (out2) {
            use = kept.y;
            if (lane == 0) ws.hcand[ci] = make_ulonglong2(kept.y, kScan);
          }
          if (use != kNoArc) {
            if (lane == 0 && use < ld_cg(&ws.best[c])) atomicMin(&ws.best[c], use);
            return;
          }
        }
        unsigned long long m = kNoArc, m2 = kNoArc;  // this lane's two lightest
        // a chunk's four 32-arc steps with their loads in flight together
        static_assert(kChunk == 4 * 32, "an MST chunk is four steps");
        uint32_t wt[4], cu[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint32_t a = b + 32 * k + lane;
          wt[k] = a < e ? __ldg(&G.w[a]) : kInf;
          cu[k] = wt[k] < kInf ? __ldg(&G.col[a]) : 0u;
          arcs += a < e;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) cu[k] = wt[k] < kInf ? ld_cg(&ws.comp[cu[k]]) : 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (wt[k] < kInf && cu[k] != c) {
            const unsigned long long key = ((unsigned long long)wt[k] << 32) | (b + 32 * k + lane);
            if (key < m) {
              m2 = m;
              m = key;
            } else if (key < m2) {
              m2 = key;
            }
          }
        }
        // the chunk's lightest, then the lightest of the rest (keys are
        // unique: one lane holds the lightest)
        const unsigned long long lo = warp_min_u64(m);
        const unsigned long long lo2 = warp_min_u64(m == lo ? m2 : m);
        if (lane == 0) {
          ws.hcand[ci] = make_ulonglong2(lo == kNoArc ? kNone : lo, lo2 == kNoArc ? kNone : lo2);
          if (lo != kNoArc) atomicMin(&ws.best[c], lo);
        }
      });
      if (!s.sync()) return;
      ++t;
    }
    // ---- B1: the root each component's lightest arc reaches
    for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
      if (ws.comp[v] != v) continue;
      const unsigned long long key = ws.best[v];
      if (key == kNoArc) continue;
      ws.partner[v] = ws.comp[__ldg(&G.col[(uint32_t)key])];
    }
    if (!s.sync()) return;
    ++t;
    // ---- B2: hook; of two roots whose arcs weigh the same, the smaller
    // stays a root (best[] stays untouched until C, so every root reads
    // its target's key)
    {
      const int cur = t % 3, old = (t + 2) % 3;
      if (leader) ws.cursor[old] = ws.hcursor[old] = ws.hooks[old] = 0;
      uint32_t hooked = 0;
      for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
        if (ws.comp[v] != v) continue;
        const unsigned long long key = ws.best[v];
        if (key == kNoArc) continue;
        const uint32_t d = ws.partner[v];
        // d is a root with an arc leaving its component (the one v chose,
        // at least), so best[d] holds a key of weight <= v's
        if ((ws.best[d] >> 32) == (key >> 32) && v < d) continue;
        ws.comp[v] = d;
        wsum += key >> 32;
        ++nedges;
        ++hooked;
        if (ws.arc_flag) ws.arc_flag[(uint32_t)key] = 1;
      }
      hooked = __reduce_add_sync(kFull, hooked);
      if (lane == 0 && hooked) atomicAdd(&ws.hooks[cur], hooked);
      if (!s.sync()) return;
      ++t;
      if (cta_words<1>([&](unsigned long long* w) { w[0] = ld_cg(&ws.hooks[cur]); })[0] == 0) break;
    }
    // ---- C: pointer jumping onto the roots; every slot starts the next
    // round empty.  Hooks form no cycle (B2), so each chase ends at a root
    // within V steps; the bound keeps the loop finite whatever happens.
    bool cycle = false;
    for (uint32_t v = W.gthread; v < G.V; v += W.nthreads) {
      ws.best[v] = kNoArc;
      uint32_t r = ld_cg(&ws.comp[v]), steps = 0;
      for (uint32_t p = ld_cg(&ws.comp[r]); p != r; p = ld_cg(&ws.comp[r])) {
        r = p;
        if (++steps > G.V) {
          cycle = true;
          break;
        }
      }
      ws.comp[v] = r;
    }
    if (cycle) atomicExch(ws.stuck, 1);
    if (!s.sync()) return;
    ++t;
    if (cta_words<1>([&](unsigned long long* w) { w[0] = (unsigned)ld_cg(ws.stuck); })[0] != 0) break;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    arcs += __shfl_xor_sync(kFull, arcs, o);
    wsum += __shfl_xor_sync(kFull, wsum, o);
    nedges += __shfl_xor_sync(kFull, nedges, o);
  }
  if (lane == 0) {
    if (wsum) atomicAdd(&ws.acc[0], wsum);
    if (nedges) atomicAdd(&ws.acc[1], nedges);
    if (arcs) atomicAdd(&ws.acc[3], arcs);
  }
  if (round > G.V && leader) *ws.stuck = 1;
  if (leader) ws.acc[2] = round + 1;
}

__global__ void __launch_bounds__(512, 3) k_mst_xf(DiscoveryArgs a, GraphView G, MstWs ws) {
  __shared__ LocalCtx l;
  __shared__ unsigned long long smem[1024];
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  mst_body(s, G, ws, smem);
}

}  // namespace

using namespace gdbi;

static int mst_run(gdb_ctx* c, gdb_graph* g, gdb_mst_result* h_res, gdb_mst_result* d_res,
                   uint8_t* d_flags) {
  if (!graph_ok(c, g)) return GDB_ERR_INVALID;
  if (!g->w) return set_error(c, GDB_ERR_INVALID, "MST needs weights");
  if (c->opt.barrier != GDB_BARRIER_XF && c->opt.barrier != GDB_BARRIER_XF_FIXED)
    return set_error(c, GDB_ERR_UNSUPPORTED, "MST runs on the XF barrier");
  const uint32_t V = g->V;
  Bump b;
  const size_t o_comp = b.take((size_t)V * 4), o_best = b.take((size_t)V * 8),
               o_part = b.take((size_t)V * 4), o_cnt = b.take(256);
  const size_t o_vc = b.take((size_t)V * 8), o_hc = b.take((size_t)std::max<uint32_t>(g->nheavy_chunks, 1) * 16);
  char* base = (char*)workspace(c, b.off);
  if (!base) return GDB_ERR_OOM;
  MstWs ws;
  ws.comp = (uint32_t*)(base + o_comp);
  ws.best = (unsigned long long*)(base + o_best);
  ws.partner = (uint32_t*)(base + o_part);
  ws.vcand = (unsigned long long*)(base + o_vc);
  ws.hcand = (ulonglong2*)(base + o_hc);
  ws.arc_flag = d_flags;
  char* cnt = base + o_cnt;
  ws.acc = (unsigned long long*)cnt;
  ws.cursor = (uint32_t*)(cnt + 64);
  ws.hcursor = (uint32_t*)(cnt + 80);
  ws.hooks = (uint32_t*)(cnt + 96);
  ws.stuck = (int*)(cnt + 112);
  const int block = c->opt.block_size;
  Shape s;
  int rc = persistent_shape(c, (const void*)k_mst_xf, block, 0, &s, c->opt.barrier == GDB_BARRIER_XF);
  if (rc) return rc;
  DiscoveryArgs a = discovery_args(c, s);
  c->last = gdb_run_stats{};
  GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  k_mst_xf<<<s.grid, block, 0, c->stream>>>(a, g->view(), ws);
  GDB_CUDA(c, cudaGetLastError());
  GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  rc = finish_run(c);
  if (rc) return rc;
  unsigned long long* hs = (unsigned long long*)pinned(c, 256);
  if (!hs) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hs, cnt, 128, cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (*(const int*)((const char*)hs + 112))
    return set_error(c, GDB_ERR_INVALID, "MST: component pointers formed a cycle");
  gdb_mst_result r;
  r.weight64 = hs[0];
  r.weight32 = (uint32_t)hs[0];
  r.edges = (uint32_t)hs[1];
  r.components = V - r.edges;
  r.rounds = (uint32_t)hs[2];
  if (h_res) *h_res = r;
  if (d_res) GDB_CUDA(c, cudaMemcpyAsync(d_res, &r, sizeof r, cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  int n = 0;
  read_participating(c, &n);
  c->last.participating = n;
  c->last.launched = s.grid;
  c->last.launches = 1;
  c->last.kernel_ms = ms;
  c->last.edges_processed = hs[3];
  c->last.supersteps = r.rounds;
  c->last.work_units = g->E;
  return GDB_OK;
}

extern "C" {

int gdb_mst_device(gdb_ctx* c, gdb_graph* g, gdb_mst_result* d_result, uint8_t* d_arc_in_mst) {
  return mst_run(c, g, nullptr, d_result, d_arc_in_mst);
}

int gdb_mst(gdb_ctx* c, gdb_graph* g, gdb_mst_result* result, uint8_t* arc_in_mst) {
  if (!graph_ok(c, g) || !result) return GDB_ERR_INVALID;
  uint8_t* d = nullptr;
  if (arc_in_mst) GDB_CUDA(c, cudaMallocAsync((void**)&d, std::max<uint64_t>(g->E, 1), c->stream));
  int rc = mst_run(c, g, result, nullptr, d);
  if (rc == GDB_OK && arc_in_mst && g->E) {
    cudaError_t e = cudaMemcpyAsync(arc_in_mst, d, g->E, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "arc flags read-back");
  }
  if (d) cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return rc;
}

}  // extern "C"
