// Host-side internals of libgdb: context, graph and launch helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "gdb.h"
#include "gdb_discovery.cuh"
#include "gdb_sweep.cuh"

// A lane: a stream with its own discovery context, barrier flags and
// workspace, so that several persistent launches of one context run at
// once (independent sources of one graph).
struct gdb_lane {
  cudaStream_t stream = nullptr;
  gdb::DeviceCtx* dctx = nullptr;
  int* flags = nullptr;
  char* ws = nullptr;
  size_t ws_bytes = 0;
};

struct gdb_ctx {
  gdb_options opt{};
  int device = 0;
  int sm_count = 0;
  int cc_major = 0, cc_minor = 0;
  size_t total_mem = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  gdb::DeviceCtx* dctx = nullptr;
  int* flags = nullptr;
  int flag_cap = 0;
  int stall_after = -1;
  unsigned long long launches = 0;  // launch ids for the XF epochs
  // grow-only device workspace
  void* ws = nullptr;
  size_t ws_bytes = 0;
  // pinned host staging for small read-backs
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  gdb_run_stats last{};
  std::string err;
  // schedule selector parameters (device copy for the kernels, host copy
  // for run-level decisions); empty = none loaded
  float* d_mlp = nullptr;
  std::vector<float> h_mlp;
  // concurrent lanes (created on first use) and, while their launches are
  // enqueued, the CTA cap each of them takes (0 = none)
  std::vector<gdb_lane> lanes;
  int cap_override = 0;
};

struct gdb_graph {
  gdb_ctx* ctx = nullptr;
  uint32_t V = 0;
  uint64_t E = 0;
  uint32_t* row = nullptr;
  uint32_t* col = nullptr;
  uint32_t* w = nullptr;
  bool owns = true;
  bool owns_w = true;
  // heavy-vertex table (degree > kHeavyDeg), ascending vertex ids
  uint32_t nheavy = 0;
  uint32_t nheavy_chunks = 0;
  uint32_t* heavy_v = nullptr;
  uint4* heavy_chunk = nullptr;    // one entry per chunk: {v, chunk, heavy index, chunks}
  uint32_t* heavy_bits = nullptr;  // V-bit membership bitmap
  double wmean = -1.0;             // mean usable weight (< 0: not measured yet)
  uint32_t wmax = 0;               // largest usable weight (with wmean)
  uint32_t maxdeg = 0;
  // light/heavy partition of the arcs for the near-far SSSP's arc split
  // (built on demand for bound split_bound; dropped with the weights)
  gdb_graph* split_l = nullptr;
  gdb_graph* split_h = nullptr;
  gdb_graph* split_t = nullptr;  // split_h transposed (in-arcs, no heavy table);
                                 // none for a graph declared symmetric
  bool symmetric = false;         // declared: u -> v (w) iff v -> u (w)
  uint32_t split_bound = 0;
  gdb::GraphView view() const;
};

namespace gdbi {

int set_cuda_error(gdb_ctx* c, cudaError_t e, const char* what);
int set_error(gdb_ctx* c, int status, const std::string& msg);

#define GDB_CUDA(c, expr)                                      \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) return gdbi::set_cuda_error(c, _e, #expr); \
  } while (0)

// Grow-only workspace; returns nullptr on failure (error recorded).
void* workspace(gdb_ctx* c, size_t bytes);
void* pinned(gdb_ctx* c, size_t bytes);

// Bump allocator over the workspace (256-byte aligned slices).
struct Bump {
  size_t off = 0;
  size_t take(size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~size_t(255);
    return o;
  }
};

// Launch shape for a persistent kernel: CTAs launched, the occupancy the
// CUDA API reports, and the discovery arguments.
struct Shape {
  int grid = 0;
  int block = 0;
  int occ_per_sm = 0;
  int fit = 0;  // occ_per_sm * sm_count
};

int persistent_shape(gdb_ctx* c, const void* kernel, int block, size_t smem, Shape* s,
                     bool allow_oversubscribe = true);
gdb::DiscoveryArgs discovery_args(gdb_ctx* c, const Shape& s);

// After a persistent run: read the device status; on error re-arm the
// discovery context and return the status.
int finish_run(gdb_ctx* c);
int reset_device_ctx(gdb_ctx* c, int skip);
// Arm a discovery context and its flags on `st` (no synchronisation).
cudaError_t arm_device_ctx(gdb_ctx* c, gdb::DeviceCtx* d, int* flags, cudaStream_t st, int skip);

// Independent runs of one graph spread over concurrent lanes: `run(lane,
// i)` enqueues run i (of n) on the lane's stream with the lane's discovery
// context and workspace (ws_bytes each); every lane takes fit / lanes CTAs
// of the kernel (fit: its co-resident CTAs on the whole GPU).  Waits for
// every lane, checks each lane's device status, records the elapsed time
// in c->last.kernel_ms.
// stats_out (optional, n x 4): the first four statistics words of each
// run's counter block (the last 512 bytes of its workspace).
// `lanes`: how many concurrent lanes (at most kMaxLanes) the n runs share;
// with `fit_memory`, fewer when the free device memory does not hold a
// workspace for each (runs whose results do not depend on the lane they
// run on: any lane count gives the same output).
int run_on_lanes(gdb_ctx* c, uint32_t n, int lanes, bool fit_memory, size_t ws_bytes, int fit,
                 const std::function<int(gdb_lane&, uint32_t)>& run,
                 unsigned long long* stats_out = nullptr);
// Discovery arguments of a launch on lane L.
gdb::DiscoveryArgs lane_args(gdb_ctx* c, const gdb_lane& L);
void lanes_destroy(gdb_ctx* c);
// Lanes of a many-source call.  R-MAT-22, 16 sources, learned schedule:
//   BFS  3.44 / 2.97 / 2.90 / 2.85 / 6.87 ms on 3 / 4 / 6 / 8 / 16 lanes,
//   SSSP 18.37 / 16.20 / 16.65 / 15.57 / 15.26 ms on the same counts
// (16 sources over 6 lanes leave two lanes short).  BC runs on 4 (gdb_bc.cu).
constexpr int kMaxLanes = 16;
constexpr int kBfsLanes = 8;
constexpr int kSsspLanes = 16;
int read_participating(gdb_ctx* c, int* n);

// Light (weight < bound) and heavy (bound <= weight < infinity) halves of
// g's arcs as two CSRs with their own heavy tables, cached on g.
int arc_split(gdb_ctx* c, gdb_graph* g, uint32_t bound);
void arc_split_drop(gdb_graph* g);

// Heavy table construction on the device from g's row array.
int build_heavy_table(gdb_graph* g);
uint32_t chunk_capacity(const gdb_graph* g);

bool graph_ok(gdb_ctx* c, gdb_graph* g);

// Device memory of graphs and their derived structures: the context
// stream's stream-ordered pool.
cudaError_t dev_alloc(gdb_ctx* c, void** p, size_t bytes);
void dev_free(gdb_ctx* c, void* p);

// Stream-capturable XF launches over a caller-owned workspace (the batch
// form): bytes of one run's workspace, and an enqueue that only issues a
// counter reset and the persistent launch on `stream`.  `proto` supplies the
// discovery context, flags, lock, timeout and release form.
// Resident CTAs per SM of the traversal kernels at `block` threads.
int traversal_occupancy(gdb_ctx* c, int block);
size_t bfs_workspace_bytes(const gdb_graph* g);
size_t sssp_workspace_bytes(const gdb_graph* g);
// `alone`: the traversal has the GPU to itself while it runs (the batch's
// one launch), not one of several sharing it (lanes, serving slots); it
// decides the automatic frontier bitmap.
int bfs_enqueue(gdb_ctx* c, gdb_graph* g, void* wsbase, const uint32_t* d_srcs, uint32_t nsrc,
                uint32_t* d_dist, cudaStream_t stream, const gdb::DiscoveryArgs& proto, bool alone);
// Allows the traversal kernels their largest shared-memory stage (once per
// context, outside any stream capture).
int bfs_prepare(gdb_ctx* c);
int sssp_enqueue(gdb_ctx* c, gdb_graph* g, void* wsbase, const uint32_t* d_srcs, uint32_t nsrc,
                 uint32_t* d_dist, cudaStream_t stream, const gdb::DiscoveryArgs& proto,
                 uint32_t delta, uint32_t light);
size_t bc_workspace_bytes(const gdb_graph* g);
int bc_enqueue(gdb_ctx* c, gdb_graph* g, void* wsbase, const uint32_t* d_sources, uint32_t nsrc,
               float* d_bc, cudaStream_t stream, const gdb::DiscoveryArgs& proto);
// Schedule of one worklist SSSP run under c's options: near-far bucket
// width (0 = label-correcting worklist), graph relaunch (when allowed) and
// the light-arc bound of the light/heavy split (GDB_LONESTAR_INF = none).
int sssp_plan(gdb_ctx* c, gdb_graph* g, uint32_t nsrc, bool allow_relaunch, uint32_t* delta,
              bool* relaunch, uint32_t* light);
// Run-level selector features of an SSSP from nsrc sources.
void sssp_features(gdb_ctx* c, const gdb_graph* g, uint32_t nsrc, float* x);

// Build, run and free a graph: init<<<grid, block>>>(G, ws, src), then a
// WHILE node whose body is level<<<grid, block>>>(G, ws, ctl, handle).
// ctl[0..1] must be zero before the launch (the init kernel leaves them).
template <class Ws>
inline int graph_while_run(gdb_ctx* c, const void* init, int grid, int block, const gdb::GraphView& G,
                           const Ws& ws, uint32_t src, const void* level, uint32_t* ctl) {
  GDB_CUDA(c, cudaMemsetAsync(ctl, 0, 8, c->stream));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaGraphCreate(&graph, 0);
  cudaGraphConditionalHandle cond = 0;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
  gdb::GraphView g0 = G;
  Ws w0 = ws;
  uint32_t s0 = src;
  uint32_t* ctl0 = ctl;
  void* init_args[] = {(void*)&g0, (void*)&w0, (void*)&s0};
  void* level_args[] = {(void*)&g0, (void*)&w0, (void*)&ctl0, (void*)&cond};
  cudaGraphNode_t n_init = nullptr, n_cond = nullptr, n_level = nullptr;
  if (e == cudaSuccess) {
    cudaKernelNodeParams kp = {};
    kp.func = (void*)init;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(block);
    kp.kernelParams = init_args;
    e = cudaGraphAddKernelNode(&n_init, graph, nullptr, 0, &kp);
  }
  cudaGraphNodeParams cp = {};
  if (e == cudaSuccess) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    e = cudaGraphAddNode(&n_cond, graph, &n_init, nullptr, 1, &cp);
  }
  if (e == cudaSuccess) {
    cudaKernelNodeParams kp = {};
    kp.func = (void*)level;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(block);
    kp.kernelParams = level_args;
    e = cudaGraphAddKernelNode(&n_level, cp.conditional.phGraph_out[0], nullptr, 0, &kp);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphUpload(exec, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev0, c->stream);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) return set_cuda_error(c, e, "graph relaunch");
  return GDB_OK;
}

}  // namespace gdbi
