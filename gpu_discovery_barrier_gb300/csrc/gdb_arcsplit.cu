// Light/heavy partition of a weighted CSR, the input of the near-far SSSP's
// arc split (the edge classes of Meyer and Sanders' delta-stepping): for a
// bound b, graph L holds every vertex's arcs of weight < b and graph H its
// arcs of weight in [b, GDB_LONESTAR_INF), each in the original order, each
// a complete CSR with its own heavy-vertex table, so the traversal kernels'
// work distribution (warp groups of light vertices, 128-arc chunks of heavy
// ones) applies to either half unchanged; graph T is H transposed (in-arcs
// and their weights, no heavy table), for pulls over heavy arcs.  Arcs of
// weight >= the infinity are never relaxed and belong to neither half.
//
// Everything is built on the device: per-vertex class counts (a warp per
// vertex of degree <= 128, a CTA per heavier vertex), exclusive scans into
// the two row arrays, an order-preserving scatter (ballot compaction), and
// the heavy tables from scans of the halves' degrees.  Only totals come
// back to the host.  The partition is cached on the graph per bound and
// dropped when its weights change.
#include <algorithm>

#include "gdb_internal.h"

namespace {

using namespace gdb;

constexpr int kScanThreads = 512;
constexpr uint32_t kScanItems = 8;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

// Exclusive scan of one value per thread over the CTA; *total gets the sum.
__device__ __forceinline__ uint32_t cta_exclusive(uint32_t x, uint32_t* total) {
  __shared__ uint32_t wsum[32];
  const int lane = lane_id(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < nw ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(kFull, s, o);
      if (lane >= o) s += t;
    }
    if (lane < nw) wsum[lane] = s;  // inclusive warp totals
  }
  __syncthreads();
  const uint32_t base = warp ? wsum[warp - 1] : 0u;
  *total = wsum[nw - 1];
  __syncthreads();
  return base + inc - x;
}

// Scan, pass 1: the sum of every tile of kScanTile items.
__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const uint32_t* in, uint32_t n,
                                                            uint32_t* sums) {
  const uint64_t t0 = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (uint32_t k = 0; k < kScanItems; ++k)
    if (t0 + k < n) s += in[t0 + k];
  uint32_t total;
  cta_exclusive(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Scan, pass 2 (one CTA): exclusive scan of the tile sums in place;
// sums[nt] = the grand total.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t* sums, uint32_t nt) {
  uint32_t carry = 0;
  for (uint32_t b = 0; b < nt; b += kScanThreads) {
    const uint32_t i = b + threadIdx.x;
    const uint32_t x = i < nt ? sums[i] : 0u;
    uint32_t total;
    const uint32_t ex = cta_exclusive(x, &total);
    if (i < nt) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) sums[nt] = carry;
}

// Scan, pass 3: out[i] = exclusive prefix of in[i]; out[n] = the total.
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* in, uint32_t n,
                                                             const uint32_t* sums, uint32_t nt,
                                                             uint32_t* out) {
  const uint64_t t0 = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems], s = 0;
#pragma unroll
  for (uint32_t k = 0; k < kScanItems; ++k) {
    v[k] = t0 + k < n ? in[t0 + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t run = sums[blockIdx.x] + cta_exclusive(s, &total);
#pragma unroll
  for (uint32_t k = 0; k < kScanItems; ++k) {
    if (t0 + k < n) out[t0 + k] = run;
    run += v[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = sums[nt];
}

__device__ __forceinline__ bool is_light(uint32_t w, uint32_t bound) { return w < bound; }
__device__ __forceinline__ bool is_heavy_arc(uint32_t w, uint32_t bound) {
  return w >= bound && w < kInf;
}

// Light and heavy arc counts of every vertex (nl, nh zeroed first: a heavy
// vertex's chunks add theirs) and of every heavy chunk (cl_c, ch_c).
__global__ void k_split_count(GraphView G, uint32_t bound, uint32_t* nl, uint32_t* nh, uint32_t* cl_c,
                              uint32_t* ch_c) {
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  const int lane = lane_id();
  // heavy vertices: one warp per 128-arc chunk, its four 32-arc steps'
  // weight loads in flight together
  for (uint32_t c = W.gwarp; c < G.nheavy_chunks; c += W.nwarps) {
    const uint4 ent = __ldg(&G.heavy_chunk[c]);
    uint32_t b, e;
    chunk_range(G, ent, b, e);
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) w[j] = b + 32 * j + lane < e ? __ldg(&G.w[b + 32 * j + lane]) : kInf;
    uint32_t cl = 0, ch = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      cl += __popc(__ballot_sync(kFull, is_light(w[j], bound)));
      ch += __popc(__ballot_sync(kFull, is_heavy_arc(w[j], bound)));
    }
    if (lane == 0) {
      cl_c[c] = cl;
      ch_c[c] = ch;
      if (cl) atomicAdd(&nl[ent.x], cl);
      if (ch) atomicAdd(&nh[ent.x], ch);
    }
  }
  // the others: 32 consecutive vertices per warp, their arcs walked together
  // four 32-arc steps at a time; the lanes of one owner in a step are found
  // with __match_any_sync and one of them adds the owner's counts
  __shared__ uint32_t scnt[2][32][32];
  uint32_t* cl_s = scnt[0][threadIdx.x >> 5];
  uint32_t* ch_s = scnt[1][threadIdx.x >> 5];
  for (uint32_t g = W.gwarp; g * 32 < G.V; g += W.nwarps) {
    const uint32_t v = g * 32 + lane;
    const bool act = v < G.V && !is_heavy(G, v);
    cl_s[lane] = ch_s[lane] = 0;
    __syncwarp();
    group_arcs4(G, act, v, [&](const bool* valid, const int* owner, const uint32_t* arc) {
      uint32_t w[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) w[j] = valid[j] ? __ldg(&G.w[arc[j]]) : kInf;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const unsigned same = __match_any_sync(kFull, owner[j]);
        const unsigned ml = __ballot_sync(kFull, valid[j] && is_light(w[j], bound)) & same;
        const unsigned mh = __ballot_sync(kFull, valid[j] && is_heavy_arc(w[j], bound)) & same;
        if (lane == 31 - __clz(same)) {
          cl_s[owner[j]] += __popc(ml);
          ch_s[owner[j]] += __popc(mh);
        }
        __syncwarp();
      }
    });
    __syncwarp();
    if (act) {
      nl[v] = cl_s[lane];
      nh[v] = ch_s[lane];
    }
    __syncwarp();
  }
}

// Order-preserving scatter of every vertex's arcs into the two halves.
__global__ void k_split_scatter(GraphView G, uint32_t bound, const uint32_t* rl, const uint32_t* rh,
                                const uint32_t* pl_c, const uint32_t* ph_c, uint32_t* cl, uint32_t* wl,
                                uint32_t* ch, uint32_t* wh) {
  const int lane = lane_id();
  // heavy vertices: one warp per 128-arc chunk; the chunk's arcs start in
  // the vertex's halves after the arcs of its earlier chunks (pl_c, ph_c:
  // exclusive scans of the per-chunk counts over the chunk table, where a
  // vertex's chunks are consecutive), so every row keeps its order
  {
    const Warps W = warps_of(blockIdx.x, gridDim.x);
    for (uint32_t c = W.gwarp; c < G.nheavy_chunks; c += W.nwarps) {
      const uint4 ent = __ldg(&G.heavy_chunk[c]);
      uint32_t b, e;
      chunk_range(G, ent, b, e);
      const uint32_t c0 = c - ent.y;  // the vertex's first chunk
      uint32_t ol = rl[ent.x] + (pl_c[c] - pl_c[c0]), oh = rh[ent.x] + (ph_c[c] - ph_c[c0]);
      uint32_t w[4], u[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t a = b + 32 * j + lane;
        w[j] = a < e ? __ldg(&G.w[a]) : kInf;
        u[j] = a < e ? __ldg(&G.col[a]) : 0u;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool il = is_light(w[j], bound), ih = is_heavy_arc(w[j], bound);
        const unsigned ml = __ballot_sync(kFull, il), mh = __ballot_sync(kFull, ih);
        if (il) {
          const uint32_t p = ol + __popc(ml & lanemask_lt());
          cl[p] = u[j];
          wl[p] = w[j];
        }
        if (ih) {
          const uint32_t p = oh + __popc(mh & lanemask_lt());
          ch[p] = u[j];
          wh[p] = w[j];
        }
        ol += __popc(ml);
        oh += __popc(mh);
      }
    }
  }
  // the others: 32 consecutive vertices per warp, four 32-arc steps at a
  // time; a lane's place in its owner's row is the owner's arcs placed so far
  // plus its rank among the owner's lanes of the step, so every row keeps
  // its order
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  __shared__ uint32_t sput[2][32][32];
  uint32_t* pl_s = sput[0][threadIdx.x >> 5];
  uint32_t* ph_s = sput[1][threadIdx.x >> 5];
  for (uint32_t g = W.gwarp; g * 32 < G.V; g += W.nwarps) {
    const uint32_t v = g * 32 + lane;
    const bool act = v < G.V && !is_heavy(G, v);
    const uint32_t ol = act ? rl[v] : 0u, oh = act ? rh[v] : 0u;
    pl_s[lane] = ph_s[lane] = 0;
    __syncwarp();
    group_arcs4(G, act, v, [&](const bool* valid, const int* owner, const uint32_t* arc) {
      uint32_t w[4], c[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        w[j] = valid[j] ? __ldg(&G.w[arc[j]]) : kInf;
        c[j] = valid[j] ? __ldg(&G.col[arc[j]]) : 0u;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const unsigned same = __match_any_sync(kFull, owner[j]);
        const bool il = valid[j] && is_light(w[j], bound), ih = valid[j] && is_heavy_arc(w[j], bound);
        const unsigned ml = __ballot_sync(kFull, il) & same, mh = __ballot_sync(kFull, ih) & same;
        const uint32_t bl = __shfl_sync(kFull, ol, owner[j]) + pl_s[owner[j]];
        const uint32_t bh = __shfl_sync(kFull, oh, owner[j]) + ph_s[owner[j]];
        if (il) {
          const uint32_t p = bl + __popc(ml & lanemask_lt());
          cl[p] = c[j];
          wl[p] = w[j];
        }
        if (ih) {
          const uint32_t p = bh + __popc(mh & lanemask_lt());
          ch[p] = c[j];
          wh[p] = w[j];
        }
        __syncwarp();
        if (lane == 31 - __clz(same)) {
          pl_s[owner[j]] += __popc(ml);
          ph_s[owner[j]] += __popc(mh);
        }
        __syncwarp();
      }
    });
    __syncwarp();
  }
}

// In-arc counts of graph H (for its transpose).
__global__ void k_in_degree(GraphView H, uint32_t* indeg) {
  for (uint64_t a = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; a < H.E;
       a += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&indeg[__ldg(&H.col[a])], 1u);
}

// Transpose of graph H: every arc u -> v (weight w) becomes v -> u in
// row v of (rt, ct, wt); fill[v] hands out the places in row v, so the
// order within a row is arbitrary.  A CTA per heavy vertex of H, a warp
// per other vertex.
__global__ void k_transpose(GraphView H, const uint32_t* rt, uint32_t* fill, uint32_t* ct,
                            uint32_t* wt) {
  auto arc = [&](uint32_t u, uint32_t a) {
    const uint32_t v = __ldg(&H.col[a]);
    const uint32_t p = rt[v] + atomicAdd(&fill[v], 1u);
    ct[p] = u;
    wt[p] = __ldg(&H.w[a]);
  };
  for (uint32_t h = blockIdx.x; h < H.nheavy; h += gridDim.x) {
    const uint32_t u = H.heavy_v[h];
    for (uint32_t a = H.row[u] + threadIdx.x; a < H.row[u + 1]; a += blockDim.x) arc(u, a);
  }
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  for (uint32_t u = W.gwarp; u < H.V; u += W.nwarps) {
    if (is_heavy(H, u)) continue;
    for (uint32_t a = H.row[u] + lane_id(); a < H.row[u + 1]; a += 32) arc(u, a);
  }
}

// Heavy-vertex marks of a CSR given by its row array: flag (degree >
// kHeavyDeg), chunk count, the membership bitmap and the largest degree.
__global__ void k_heavy_marks(const uint32_t* row, uint32_t V, uint32_t* flag, uint32_t* nch,
                              uint32_t* bits, uint32_t* maxdeg) {
  const Warps W = warps_of(blockIdx.x, gridDim.x);
  const int lane = lane_id();
  uint32_t md = 0;
  for (uint32_t base = W.gwarp * 32; base < V; base += W.nwarps * 32) {
    const uint32_t v = base + lane;
    const uint32_t d = v < V ? row[v + 1] - row[v] : 0u;
    const bool hv = d > kHeavyDeg;
    if (v < V) {
      flag[v] = hv;
      nch[v] = hv ? chunks_of(d) : 0u;
    }
    const unsigned m = __ballot_sync(kFull, hv);
    if (lane == 0) bits[base >> 5] = m;
    md = max(md, d);
  }
  md = __reduce_max_sync(kFull, md);
  if (lane == 0 && md) atomicMax(maxdeg, md);
}

// Heavy vertex list and chunk entries {vertex, chunk, heavy index, chunks}.
__global__ void k_heavy_fill(const uint32_t* row, uint32_t V, const uint32_t* flag,
                             const uint32_t* hidx, const uint32_t* cbase, uint32_t* heavy_v,
                             uint4* chunks) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    if (!flag[v]) continue;
    const uint32_t h = hidx[v], n = chunks_of(row[v + 1] - row[v]), cb = cbase[v];
    heavy_v[h] = v;
    for (uint32_t j = 0; j < n; ++j) chunks[cb + j] = make_uint4(v, j, h, n);
  }
}

}  // namespace

namespace gdbi {

// out[0..n] = exclusive scan of in[0..n) and the total; `tmp` holds
// scan_tmp_words(n) words.
static uint32_t scan_tiles(uint32_t n) { return std::max<uint32_t>((n + kScanTile - 1) / kScanTile, 1); }
static size_t scan_tmp_words(uint32_t n) { return (size_t)scan_tiles(n) + 1; }

static cudaError_t exclusive_scan(const uint32_t* in, uint32_t n, uint32_t* out, uint32_t* tmp,
                                  cudaStream_t st) {
  const uint32_t nt = scan_tiles(n);
  k_tile_sums<<<nt, kScanThreads, 0, st>>>(in, n, tmp);
  k_scan_sums<<<1, kScanThreads, 0, st>>>(tmp, nt);
  k_scan_tiles<<<nt, kScanThreads, 0, st>>>(in, n, tmp, nt, out);
  return cudaGetLastError();
}

void arc_split_drop(gdb_graph* g) {
  if (g->split_l) gdb_graph_destroy(g->split_l);
  if (g->split_h) gdb_graph_destroy(g->split_h);
  if (g->split_t) gdb_graph_destroy(g->split_t);
  g->split_l = g->split_h = g->split_t = nullptr;
  g->split_bound = 0;
}

// Heavy table of a derived CSR whose row array is on the device; `t0`,
// `t1` (V + 1 words each) and `tmp` are scratch.
static int heavy_table_device(gdb_ctx* c, gdb_graph* x, uint32_t* t0, uint32_t* t1, uint32_t* t2,
                              uint32_t* t3, uint32_t* tmp, uint32_t* hs) {
  const uint32_t V = x->V;
  cudaStream_t st = c->stream;
  const size_t nb = ((size_t)(V + 31) / 32 + 1) * 4;
  GDB_CUDA(c, dev_alloc(c, (void**)&x->heavy_bits, nb));
  GDB_CUDA(c, cudaMemsetAsync(x->heavy_bits, 0, nb, st));
  GDB_CUDA(c, cudaMemsetAsync(hs, 0, 16, st));
  const int grid = 8 * c->sm_count;  // every 256-thread CTA resident: the loops are latency-bound
  k_heavy_marks<<<grid, 256, 0, st>>>(x->row, V, t0, t1, x->heavy_bits, hs + 2);
  GDB_CUDA(c, cudaGetLastError());
  GDB_CUDA(c, exclusive_scan(t0, V, t2, tmp, st));
  GDB_CUDA(c, exclusive_scan(t1, V, t3, tmp, st));
  GDB_CUDA(c, cudaMemcpyAsync(hs, t2 + V, 4, cudaMemcpyDeviceToDevice, st));
  GDB_CUDA(c, cudaMemcpyAsync(hs + 1, t3 + V, 4, cudaMemcpyDeviceToDevice, st));
  uint32_t* hh = (uint32_t*)pinned(c, 64);
  if (!hh) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemcpyAsync(hh, hs, 12, cudaMemcpyDeviceToHost, st));
  GDB_CUDA(c, cudaStreamSynchronize(st));
  x->nheavy = hh[0];
  x->nheavy_chunks = hh[1];
  x->maxdeg = hh[2];
  GDB_CUDA(c, dev_alloc(c, (void**)&x->heavy_v, std::max<size_t>(x->nheavy, 1) * 4));
  GDB_CUDA(c, dev_alloc(c, (void**)&x->heavy_chunk, std::max<size_t>(x->nheavy_chunks, 1) * sizeof(uint4)));
  k_heavy_fill<<<grid, 256, 0, st>>>(x->row, V, t0, t2, t3, x->heavy_v, x->heavy_chunk);
  GDB_CUDA(c, cudaGetLastError());
  return GDB_OK;
}

// One pass over a CSR's arrays: bit 0 when a row pointer decreases, bit 1
// when a column names a vertex >= V -- a graph every kernel would read or
// write out of bounds.
__global__ void k_check_csr(const uint32_t* __restrict__ row, const uint32_t* __restrict__ col, uint32_t V,
                            uint64_t E, uint32_t* bad) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t b = 0;
  for (uint64_t i = t0; i < V; i += stride) b |= __ldg(&row[i + 1]) < __ldg(&row[i]) ? 1u : 0u;
  for (uint64_t e = t0; e < E; e += stride) b |= __ldg(&col[e]) >= V ? 2u : 0u;
  b = __reduce_or_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0 && b) atomicOr(bad, b);
}

// The heavy table of a graph whose row array is on the device (every graph
// the library creates): scratch of its own, one synchronisation for the
// CSR check and one for the totals.  The check runs first: the table's
// degrees come from the row array.
int build_heavy_table(gdb_graph* g) {
  gdb_ctx* c = g->ctx;
  const uint32_t V = g->V;
  const size_t vw = (size_t)V + 1;
  uint32_t* scratch = nullptr;
  GDB_CUDA(c, cudaMallocAsync((void**)&scratch, (4 * vw + scan_tmp_words(V) + 8) * 4, c->stream));
  uint32_t *t0 = scratch, *t1 = t0 + vw, *t2 = t1 + vw, *t3 = t2 + vw, *tmp = t3 + vw,
           *hs = tmp + scan_tmp_words(V);
  uint32_t bad = 0;
  cudaError_t ce = cudaMemsetAsync(hs + 7, 0, 4, c->stream);
  if (ce == cudaSuccess) {
    k_check_csr<<<4 * std::max(c->sm_count, 1), 256, 0, c->stream>>>(g->row, g->col, V, g->E, hs + 7);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&bad, hs + 7, 4, cudaMemcpyDeviceToHost, c->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
  if (ce != cudaSuccess || bad) {
    cudaFreeAsync(scratch, c->stream);
    cudaStreamSynchronize(c->stream);
    if (ce != cudaSuccess) return set_cuda_error(c, ce, "CSR check");
    return set_error(c, GDB_ERR_INVALID, (bad & 1) ? "row_ptr decreases" : "a column names a vertex >= V");
  }
  const int rc = heavy_table_device(c, g, t0, t1, t2, t3, tmp, hs);
  cudaFreeAsync(scratch, c->stream);
  const cudaError_t e = cudaStreamSynchronize(c->stream);
  if (rc) return rc;
  return e == cudaSuccess ? GDB_OK : set_cuda_error(c, e, "heavy table");
}

static gdb_graph* new_half(gdb_ctx* c, uint32_t V) {
  gdb_graph* x = new gdb_graph();
  x->ctx = c;
  x->V = V;
  return x;
}

int arc_split(gdb_ctx* c, gdb_graph* g, uint32_t bound) {
  if (!g->w) return set_error(c, GDB_ERR_INVALID, "arc split needs weights");
  if (g->split_l && g->split_bound == bound) return GDB_OK;
  arc_split_drop(g);
  const uint32_t V = g->V;
  cudaStream_t st = c->stream;
  gdb_graph* L = new_half(c, V);
  gdb_graph* H = new_half(c, V);
  gdb_graph* T = nullptr;  // transpose of H, built last
  // scratch: four V + 1 word arrays, the scan's tile sums, totals, and
  // four arrays over the heavy chunks (counts and their scans)
  const size_t vw = (size_t)V + 1;
  const uint32_t nch = g->nheavy_chunks;
  const size_t cw = (size_t)nch + 1;
  uint32_t* scratch = nullptr;
  const size_t words = 4 * vw + std::max(scan_tmp_words(V), scan_tmp_words(nch)) + 8 + 4 * cw;
  int rc = GDB_OK;
  auto fail = [&](int r) {
    if (scratch) cudaFreeAsync(scratch, st);
    cudaStreamSynchronize(st);
    gdb_graph_destroy(L);
    gdb_graph_destroy(H);
    if (T) gdb_graph_destroy(T);
    return r;
  };
  cudaError_t e = cudaMallocAsync((void**)&scratch, words * 4, st);
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "arc split scratch"));
  uint32_t *t0 = scratch, *t1 = t0 + vw, *t2 = t1 + vw, *t3 = t2 + vw, *tmp = t3 + vw,
           *hs = tmp + std::max(scan_tmp_words(V), scan_tmp_words(nch)), *cl_c = hs + 8, *ch_c = cl_c + cw,
           *pl_c = ch_c + cw, *ph_c = pl_c + cw;
  e = dev_alloc(c, (void**)&L->row, vw * 4);
  if (e == cudaSuccess) e = dev_alloc(c, (void**)&H->row, vw * 4);
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "arc split rows"));
  const GraphView G = g->view();
  const int grid = 8 * c->sm_count;  // every 256-thread CTA resident: the loops are latency-bound
  // a heavy vertex's counts are added up over its chunks
  e = cudaMemsetAsync(t0, 0, 2 * vw * 4, st);
  if (e == cudaSuccess) {
    k_split_count<<<grid, 256, 0, st>>>(G, bound, t0, t1, cl_c, ch_c);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = exclusive_scan(t0, V, L->row, tmp, st);
  if (e == cudaSuccess) e = exclusive_scan(t1, V, H->row, tmp, st);
  if (e == cudaSuccess && nch) e = exclusive_scan(cl_c, nch, pl_c, tmp, st);
  if (e == cudaSuccess && nch) e = exclusive_scan(ch_c, nch, ph_c, tmp, st);
  uint32_t* hh = (uint32_t*)pinned(c, 64);
  if (!hh) return fail(GDB_ERR_OOM);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hh, L->row + V, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hh + 1, H->row + V, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "arc split counts"));
  L->E = hh[0];
  H->E = hh[1];
  e = dev_alloc(c, (void**)&L->col, std::max<uint64_t>(L->E, 1) * 4);
  if (e == cudaSuccess) e = dev_alloc(c, (void**)&L->w, std::max<uint64_t>(L->E, 1) * 4);
  if (e == cudaSuccess) e = dev_alloc(c, (void**)&H->col, std::max<uint64_t>(H->E, 1) * 4);
  if (e == cudaSuccess) e = dev_alloc(c, (void**)&H->w, std::max<uint64_t>(H->E, 1) * 4);
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "arc split arcs"));
  k_split_scatter<<<grid, 256, 0, st>>>(G, bound, L->row, H->row, pl_c, ph_c, L->col, L->w, H->col, H->w);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "arc split scatter"));
  if ((rc = heavy_table_device(c, L, t0, t1, t2, t3, tmp, hs))) return fail(rc);
  if ((rc = heavy_table_device(c, H, t0, t1, t2, t3, tmp, hs))) return fail(rc);
  // the transpose of the heavy half: in-arcs with their weights, for the
  // pull form of a settle superstep -- a graph declared symmetric (with
  // symmetric weights) is its own transpose
  if (!g->symmetric) {
    T = new_half(c, V);
    T->E = H->E;
    e = dev_alloc(c, (void**)&T->row, vw * 4);
    if (e == cudaSuccess) e = dev_alloc(c, (void**)&T->col, std::max<uint64_t>(T->E, 1) * 4);
    if (e == cudaSuccess) e = dev_alloc(c, (void**)&T->w, std::max<uint64_t>(T->E, 1) * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(t0, 0, vw * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(t1, 0, vw * 4, st);
    if (e != cudaSuccess) return fail(set_cuda_error(c, e, "arc split transpose"));
    const GraphView HV = H->view();
    k_in_degree<<<grid, 256, 0, st>>>(HV, t0);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = exclusive_scan(t0, V, T->row, tmp, st);
    if (e == cudaSuccess) {
      k_transpose<<<grid, 256, 0, st>>>(HV, T->row, t1, T->col, T->w);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return fail(set_cuda_error(c, e, "arc split transpose"));
  }
  cudaFreeAsync(scratch, st);
  e = cudaStreamSynchronize(st);
  scratch = nullptr;
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "arc split"));
  g->split_l = L;
  g->split_h = H;
  g->split_t = T;
  g->split_bound = bound;
  return GDB_OK;
}

}  // namespace gdbi
