// Batched form: many graphs, one BFS and one SSSP query each, as two
// persistent launches captured once into a CUDA graph.
//
// The graphs are packed into one disjoint-union CSR (graph i's vertices are
// [vertex_offset[i], vertex_offset[i+1])).  No arc crosses two graphs, so a
// multi-source traversal from one source per graph computes every graph's
// own answer: a vertex can only be reached from its own graph's source, and
// its level / distance is the one of the single-graph run.  The union's
// frontier holds all graphs' frontiers at once; the persistent kernel
// balances arcs across every CTA regardless of which graph they belong to,
// and the whole batch takes max(levels) barrier intervals instead of
// sum(levels) launches.
//
// A batch owns its workspace, its discovery context and its barrier flags,
// so its graph replays on the context's stream without touching the
// context's own device state.  The captured launches use the counting XF
// forms (flat or combining by participant count), which need no
// launch-unique epoch -- combining arrival counts are zeroed when a launch
// ends and its release generation only changes; the flat count carries
// over from launch to launch through the context -- so they are valid on
// every replay.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "gdb_internal.h"

using namespace gdbi;

struct gdb_batch {
  gdb_ctx* ctx = nullptr;
  gdb_graph* g = nullptr;
  uint32_t apps = 0;
  uint32_t nsrc = 0;
  gdb::DeviceCtx* dctx = nullptr;
  int* flags = nullptr;
  char* mem = nullptr;        // one device allocation: results, sources, workspaces
  uint32_t* d_bfs = nullptr;
  uint32_t* d_sssp = nullptr;
  uint32_t* d_srcs = nullptr;
  char* ws_bfs = nullptr;
  char* ws_sssp = nullptr;
  size_t cnt_off_bfs = 0, cnt_off_sssp = 0;  // counter blocks inside the workspaces
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint32_t delta = 0;         // near-far bucket width of the SSSP launch
  uint32_t light = GDB_LONESTAR_INF;  // its light-arc bound (split when < inf)
  unsigned long long host_stats[2][8] = {};
};

static int batch_arm(gdb_batch* b) {
  gdb_ctx* c = b->ctx;
  gdb::DeviceCtx h;
  std::memset(&h, 0, sizeof(h));
  h.poll_open = 1;
  h.stall_after = -1;
  GDB_CUDA(c, cudaMemcpyAsync(b->dctx, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaMemsetAsync(b->flags, 0, (size_t)c->flag_cap * gdb::kLineInts * sizeof(int), c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  return GDB_OK;
}

extern "C" {

int gdb_graph_create_batch(gdb_ctx* c, uint32_t n, const uint32_t* V, const uint64_t* E,
                           const uint32_t* const* row_ptr, const uint32_t* const* col,
                           const uint32_t* const* w, uint32_t* vertex_offset, gdb_graph** out) {
  if (!c || !out || n == 0 || !V || !E || !row_ptr || !col) return GDB_ERR_INVALID;
  uint64_t Vt = 0, Et = 0;
  for (uint32_t i = 0; i < n; ++i) {
    if (!row_ptr[i] || (E[i] && !col[i]) || (w && E[i] && !w[i])) return GDB_ERR_INVALID;
    if (row_ptr[i][0] != 0 || row_ptr[i][V[i]] != E[i])
      return set_error(c, GDB_ERR_INVALID, "batch member row_ptr does not span its arcs");
    Vt += V[i];
    Et += E[i];
  }
  if (Vt >= (1ull << 31) || Et >= (1ull << 32))
    return set_error(c, GDB_ERR_INVALID, "batch union exceeds V < 2^31, E < 2^32");
  std::vector<uint32_t> row((size_t)Vt + 1), cl((size_t)Et), wt(w ? (size_t)Et : 0);
  uint64_t vo = 0, eo = 0;
  for (uint32_t i = 0; i < n; ++i) {
    if (vertex_offset) vertex_offset[i] = (uint32_t)vo;
    for (uint32_t v = 0; v < V[i]; ++v) row[vo + v] = (uint32_t)(eo + row_ptr[i][v]);
    for (uint64_t e = 0; e < E[i]; ++e) {
      const uint32_t d = col[i][e];
      if (d >= V[i]) return set_error(c, GDB_ERR_INVALID, "batch member arc out of range");
      cl[eo + e] = (uint32_t)(vo + d);
    }
    if (w && E[i]) std::memcpy(&wt[eo], w[i], E[i] * 4);
    vo += V[i];
    eo += E[i];
  }
  row[Vt] = (uint32_t)Et;
  if (vertex_offset) vertex_offset[n] = (uint32_t)Vt;
  return gdb_graph_create(c, (uint32_t)Vt, Et, row.data(), cl.data(), w ? wt.data() : nullptr, out);
}

int gdb_batch_destroy(gdb_batch* b) {
  if (!b) return GDB_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->mem) cudaFree(b->mem);
  if (b->flags) cudaFree(b->flags);
  if (b->dctx) cudaFree(b->dctx);
  delete b;
  return GDB_OK;
}

int gdb_batch_create(gdb_ctx* c, gdb_graph* g, uint32_t apps, const uint32_t* sources, uint32_t nsrc,
                     gdb_batch** out) {
  if (!out || !graph_ok(c, g) || !sources || nsrc == 0) return GDB_ERR_INVALID;
  *out = nullptr;
  if (apps == 0 || (apps & ~(GDB_BATCH_BFS | GDB_BATCH_SSSP)))
    return set_error(c, GDB_ERR_INVALID, "batch apps must be a non-empty mask of BFS and SSSP");
  if ((apps & GDB_BATCH_SSSP) && !g->w) return set_error(c, GDB_ERR_INVALID, "SSSP needs weights");
  for (uint32_t i = 0; i < nsrc; ++i)
    if (sources[i] >= g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  gdb_batch* b = new gdb_batch;
  b->ctx = c;
  b->g = g;
  b->apps = apps;
  b->nsrc = nsrc;
  int rc = GDB_OK;
  auto fail = [&](int r) {
    gdb_batch_destroy(b);
    return r;
  };
  // device memory: [bfs dist][sssp dist][sources][bfs ws][sssp ws]
  Bump m;
  const size_t vb = (size_t)g->V * 4;
  const size_t o_bfs = m.take(vb), o_sssp = m.take(vb), o_src = m.take((size_t)nsrc * 4);
  const size_t o_wb = m.take((apps & GDB_BATCH_BFS) ? bfs_workspace_bytes(g) : 0);
  const size_t o_ws = m.take((apps & GDB_BATCH_SSSP) ? sssp_workspace_bytes(g) : 0);
  cudaError_t e = cudaMalloc((void**)&b->mem, m.off);
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->dctx, sizeof(gdb::DeviceCtx));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->flags, (size_t)c->flag_cap * gdb::kLineInts * sizeof(int));
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? set_error(c, GDB_ERR_OOM, "batch workspace")
                                                                   : set_cuda_error(c, e, "batch create"));
  b->d_bfs = (uint32_t*)(b->mem + o_bfs);
  b->d_sssp = (uint32_t*)(b->mem + o_sssp);
  b->d_srcs = (uint32_t*)(b->mem + o_src);
  b->ws_bfs = b->mem + o_wb;
  b->ws_sssp = b->mem + o_ws;
  e = cudaMemcpyAsync(b->d_srcs, sources, (size_t)nsrc * 4, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "batch sources"));
  if ((rc = batch_arm(b))) return fail(rc);
  bool relaunch = false;
  if ((apps & GDB_BATCH_SSSP) && (rc = sssp_plan(c, g, nsrc, false, &b->delta, &relaunch, &b->light))) return fail(rc);

  gdb::DiscoveryArgs proto;
  proto.ctx = b->dctx;
  proto.flags = b->flags;
  proto.flag_capacity = c->flag_cap;
  proto.lock_kind = c->opt.lock;
  proto.expected = 0;
  proto.timeout_ns = c->opt.timeout_ns ? c->opt.timeout_ns : 2000000000ull;
  proto.close_wait_ns = 50000ull;
  proto.launch_id = 1;
  proto.xf_release = gdb::kXfAuto;

  cudaStream_t cs = nullptr;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "capture stream"));
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    if (apps & GDB_BATCH_BFS) rc = bfs_enqueue(c, g, b->ws_bfs, b->d_srcs, nsrc, b->d_bfs, cs, proto, true);
    if (rc == GDB_OK && (apps & GDB_BATCH_SSSP))
      rc = sssp_enqueue(c, g, b->ws_sssp, b->d_srcs, nsrc, b->d_sssp, cs, proto, b->delta, b->light);
    cudaError_t e2 = cudaStreamEndCapture(cs, &b->graph);
    if (rc == GDB_OK && e2 != cudaSuccess) rc = set_cuda_error(c, e2, "batch capture");
  } else {
    rc = set_cuda_error(c, e, "batch capture");
  }
  cudaStreamDestroy(cs);
  if (rc) return fail(rc);
  e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e == cudaSuccess) e = cudaGraphUpload(b->exec, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(set_cuda_error(c, e, "batch instantiate"));
  // counter blocks sit at the end of each workspace (last 512-byte slice)
  if (apps & GDB_BATCH_BFS) b->cnt_off_bfs = bfs_workspace_bytes(g) - 512;
  if (apps & GDB_BATCH_SSSP) b->cnt_off_sssp = sssp_workspace_bytes(g) - 512;
  *out = b;
  return GDB_OK;
}

int gdb_batch_set_sources(gdb_batch* b, const uint32_t* sources) {
  if (!b || !sources) return GDB_ERR_INVALID;
  gdb_ctx* c = b->ctx;
  for (uint32_t i = 0; i < b->nsrc; ++i)
    if (sources[i] >= b->g->V) return set_error(c, GDB_ERR_INVALID, "source out of range");
  GDB_CUDA(c, cudaMemcpyAsync(b->d_srcs, sources, (size_t)b->nsrc * 4, cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  return GDB_OK;
}

int gdb_batch_launch(gdb_batch* b) {
  if (!b) return GDB_ERR_INVALID;
  gdb_ctx* c = b->ctx;
  GDB_CUDA(c, cudaEventRecord(b->ev0, c->stream));
  GDB_CUDA(c, cudaGraphLaunch(b->exec, c->stream));
  GDB_CUDA(c, cudaEventRecord(b->ev1, c->stream));
  return GDB_OK;
}

int gdb_batch_wait(gdb_batch* b, double* ms) {
  if (!b) return GDB_ERR_INVALID;
  gdb_ctx* c = b->ctx;
  char* hp = (char*)pinned(c, 4096);
  if (!hp) return GDB_ERR_OOM;
  int* h = (int*)(hp + 3584);
  unsigned long long* hs = (unsigned long long*)hp;  // [0, 1024): two counter blocks
  GDB_CUDA(c, cudaMemcpyAsync(h, &b->dctx->status, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (b->apps & GDB_BATCH_BFS)
    GDB_CUDA(c, cudaMemcpyAsync(hs, b->ws_bfs + b->cnt_off_bfs, 512, cudaMemcpyDeviceToHost, c->stream));
  if (b->apps & GDB_BATCH_SSSP)
    GDB_CUDA(c, cudaMemcpyAsync(hs + 64, b->ws_sssp + b->cnt_off_sssp, 512, cudaMemcpyDeviceToHost,
                                c->stream));
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return set_cuda_error(c, e, "batch execution");
  if (h[0] != 0) {
    const int status = h[0], where = h[2];
    batch_arm(b);
    char buf[160];
    snprintf(buf, sizeof buf, "batch: device reported %s at site %d", gdb_status_string(status), where);
    c->err = buf;
    return status;
  }
  for (int a = 0; a < 2; ++a) {
    if (!(b->apps & (1u << a))) continue;
    const unsigned long long* s = hs + 64 * a;
    if (*(const int*)((const char*)s + 160)) return set_error(c, GDB_ERR_CAPACITY, "batch queue overflow");
    std::memcpy(b->host_stats[a], s, 64);
  }
  float t = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&t, b->ev0, b->ev1));
  if (ms) *ms = t;
  c->last = gdb_run_stats{};
  c->last.kernel_ms = t;
  c->last.launches = __builtin_popcount(b->apps);
  c->last.edges_processed = b->host_stats[0][0] + b->host_stats[1][0];
  c->last.supersteps = (uint32_t)(b->host_stats[0][1] + b->host_stats[1][1]);
  return GDB_OK;
}

int gdb_batch_run(gdb_batch* b, double* ms) {
  int rc = gdb_batch_launch(b);
  return rc ? rc : gdb_batch_wait(b, ms);
}

int gdb_batch_results(gdb_batch* b, uint32_t* bfs_dist, uint32_t* sssp_dist) {
  if (!b) return GDB_ERR_INVALID;
  gdb_ctx* c = b->ctx;
  const size_t vb = (size_t)b->g->V * 4;
  if (bfs_dist) {
    if (!(b->apps & GDB_BATCH_BFS)) return set_error(c, GDB_ERR_INVALID, "BFS not in this batch");
    GDB_CUDA(c, cudaMemcpyAsync(bfs_dist, b->d_bfs, vb, cudaMemcpyDeviceToHost, c->stream));
  }
  if (sssp_dist) {
    if (!(b->apps & GDB_BATCH_SSSP)) return set_error(c, GDB_ERR_INVALID, "SSSP not in this batch");
    GDB_CUDA(c, cudaMemcpyAsync(sssp_dist, b->d_sssp, vb, cudaMemcpyDeviceToHost, c->stream));
  }
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  return GDB_OK;
}

const uint32_t* gdb_batch_device_result(gdb_batch* b, uint32_t app) {
  if (!b || !(b->apps & app)) return nullptr;
  return app == GDB_BATCH_BFS ? b->d_bfs : app == GDB_BATCH_SSSP ? b->d_sssp : nullptr;
}

int gdb_batch_app_stats(gdb_batch* b, uint32_t app, uint64_t* arcs, uint32_t* supersteps) {
  if (!b || (app != GDB_BATCH_BFS && app != GDB_BATCH_SSSP) || !(b->apps & app)) return GDB_ERR_INVALID;
  const int a = app == GDB_BATCH_BFS ? 0 : 1;
  if (arcs) *arcs = b->host_stats[a][0];
  if (supersteps) *supersteps = (uint32_t)b->host_stats[a][1];
  return GDB_OK;
}

}  // extern "C"
