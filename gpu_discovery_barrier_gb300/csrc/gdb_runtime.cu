// libgdb host runtime: contexts, graphs, workspace, launch shapes, errors.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "gdb_internal.h"

namespace gdbi {

int set_cuda_error(gdb_ctx* c, cudaError_t e, const char* what) {
  if (c) {
    c->err = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  }
  cudaGetLastError();  // clear the sticky-free error so the context stays usable
  return e == cudaErrorMemoryAllocation ? GDB_ERR_OOM : GDB_ERR_CUDA;
}

int set_error(gdb_ctx* c, int status, const std::string& msg) {
  if (c) c->err = msg;
  return status;
}

void* workspace(gdb_ctx* c, size_t bytes) {
  if (bytes <= c->ws_bytes) return c->ws;
  if (c->ws) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->ws);
    c->ws = nullptr;
    c->ws_bytes = 0;
  }
  size_t want = std::max(bytes, (size_t)1 << 20);
  cudaError_t e = cudaMalloc(&c->ws, want);
  if (e != cudaSuccess) {
    set_cuda_error(c, e, "cudaMalloc(workspace)");
    c->ws = nullptr;
    return nullptr;
  }
  c->ws_bytes = want;
  return c->ws;
}

void* pinned(gdb_ctx* c, size_t bytes) {
  if (bytes <= c->pinned_bytes) return c->pinned;
  if (c->pinned) cudaFreeHost(c->pinned);
  c->pinned = nullptr;
  c->pinned_bytes = 0;
  size_t want = std::max(bytes, (size_t)4096);
  if (cudaMallocHost(&c->pinned, want) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  c->pinned_bytes = want;
  return c->pinned;
}

int persistent_shape(gdb_ctx* c, const void* kernel, int block, size_t smem, Shape* s,
                     bool allow_oversubscribe) {
  int occ = 0;
  GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, block, smem));
  if (occ <= 0) return set_error(c, GDB_ERR_INVALID, "kernel does not fit on an SM at this block size");
  s->block = block;
  s->occ_per_sm = occ;
  s->fit = occ * c->sm_count;
  int grid = s->fit;
  if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
  if (c->cap_override > 0) grid = std::min(grid, c->cap_override);  // a lane's share
  if (allow_oversubscribe && c->opt.oversubscribe > 0) grid = c->opt.oversubscribe;
  // the XF master retires at most 32 peers per thread; flags bound P
  const int cap = std::min(c->flag_cap, 32 * block + 1);
  if (!(allow_oversubscribe && c->opt.oversubscribe > 0)) grid = std::min(grid, cap);
  s->grid = std::max(grid, 1);
  return GDB_OK;
}

gdb::DiscoveryArgs discovery_args(gdb_ctx* c, const Shape& s) {
  gdb::DiscoveryArgs a;
  a.ctx = c->dctx;
  a.flags = c->flags;
  a.flag_capacity = c->flag_cap;
  a.lock_kind = c->opt.lock;
  a.expected = std::min(s.grid, s.fit);
  a.timeout_ns = c->opt.timeout_ns ? c->opt.timeout_ns : 2000000000ull;
  a.close_wait_ns = 50000ull;
  a.launch_id = ++c->launches;
  a.xf_release = c->opt.xf_release;
  return a;
}

cudaError_t arm_device_ctx(gdb_ctx* c, gdb::DeviceCtx* d, int* flags, cudaStream_t st, int skip) {
  gdb::DeviceCtx h;
  std::memset(&h, 0, sizeof(h));
  h.poll_open = 1;
  h.skip = skip;
  h.stall_after = c->stall_after;
  // pageable source: the copy has taken h before the call returns
  cudaError_t e = cudaMemcpyAsync(d, &h, sizeof(h), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(flags, 0, (size_t)c->flag_cap * gdb::kLineInts * sizeof(int), st);
  return e;
}

int reset_device_ctx(gdb_ctx* c, int skip) {
  GDB_CUDA(c, arm_device_ctx(c, c->dctx, c->flags, c->stream, skip));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  return GDB_OK;
}

void lanes_destroy(gdb_ctx* c) {
  for (gdb_lane& L : c->lanes) {
    if (L.stream) cudaStreamSynchronize(L.stream);
    cudaFree(L.ws);
    cudaFree(L.dctx);
    cudaFree(L.flags);
    if (L.stream) cudaStreamDestroy(L.stream);
  }
  c->lanes.clear();
  cudaGetLastError();
}

gdb::DiscoveryArgs lane_args(gdb_ctx* c, const gdb_lane& L) {
  gdb::DiscoveryArgs a;
  a.ctx = L.dctx;
  a.flags = L.flags;
  a.flag_capacity = c->flag_cap;
  a.lock_kind = c->opt.lock;
  a.expected = 0;
  a.timeout_ns = c->opt.timeout_ns ? c->opt.timeout_ns : 2000000000ull;
  a.close_wait_ns = 50000ull;
  a.launch_id = ++c->launches;
  a.xf_release = c->opt.xf_release;
  return a;
}

int run_on_lanes(gdb_ctx* c, uint32_t n, int lanes, bool fit_memory, size_t ws_bytes, int fit,
                 const std::function<int(gdb_lane&, uint32_t)>& run,
                 unsigned long long* stats_out) {
  int k = (int)std::min<uint32_t>((uint32_t)std::min(std::max(lanes, 1), kMaxLanes),
                                  std::max<uint32_t>(n, 1u));
  if (fit_memory && k > 1) {
    // lanes that already hold a large enough workspace, plus as many new
    // ones as half of the free device memory holds (at least one lane)
    int ready = 0;
    for (int i = 0; i < (int)c->lanes.size() && i < k; ++i) ready += c->lanes[i].ws_bytes >= ws_bytes;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && ws_bytes > 0) {
      const size_t more = free_b / 2 / ws_bytes;
      k = std::max(1, (int)std::min<size_t>((size_t)k, (size_t)ready + more));
    } else {
      cudaGetLastError();
    }
  }
  while ((int)c->lanes.size() < k) {
    gdb_lane L;
    cudaError_t e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&L.dctx, sizeof(gdb::DeviceCtx));
    if (e == cudaSuccess) e = cudaMalloc(&L.flags, (size_t)c->flag_cap * gdb::kLineInts * sizeof(int));
    if (e == cudaSuccess) e = arm_device_ctx(c, L.dctx, L.flags, L.stream, 0);
    if (e != cudaSuccess) {
      c->lanes.push_back(L);  // freed with the others
      lanes_destroy(c);
      return set_cuda_error(c, e, "lane creation");
    }
    c->lanes.push_back(L);
  }
  for (int i = 0; i < k; ++i) {
    gdb_lane& L = c->lanes[i];
    if (L.ws_bytes < ws_bytes) {
      GDB_CUDA(c, cudaStreamSynchronize(L.stream));
      cudaFree(L.ws);
      L.ws = nullptr;
      L.ws_bytes = 0;
      GDB_CUDA(c, cudaMalloc(&L.ws, ws_bytes));
      L.ws_bytes = ws_bytes;
    }
  }
  // per run: its 32 statistics bytes and overflow word, read back after
  unsigned long long* stage = (unsigned long long*)pinned(c, 4096 + (size_t)n * 64);
  if (!stage) return GDB_ERR_OOM;
  stage += 512;  // past the staging the single runs use
  // the lanes start after the work already queued on the context's stream
  GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  for (int i = 0; i < k; ++i) GDB_CUDA(c, cudaStreamWaitEvent(c->lanes[i].stream, c->ev0, 0));
  c->cap_override = std::max(1, fit / k);
  int rc = GDB_OK;
  for (uint32_t i = 0; i < n && rc == GDB_OK; ++i) {
    gdb_lane& L = c->lanes[i % k];
    rc = run(L, i);
    const char* cnt = L.ws + ws_bytes - 512;
    if (rc == GDB_OK) {
      cudaError_t e = cudaMemcpyAsync(stage + 8 * i, cnt, 32, cudaMemcpyDeviceToHost, L.stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(stage + 8 * i + 4, cnt + 160, 4, cudaMemcpyDeviceToHost, L.stream);
      if (e != cudaSuccess) rc = set_cuda_error(c, e, "lane statistics");
    }
  }
  c->cap_override = 0;
  // join: the context's stream waits for every lane
  for (int i = 0; i < k; ++i) {
    gdb_lane& L = c->lanes[i];
    cudaEvent_t done;
    GDB_CUDA(c, cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    cudaEventRecord(done, L.stream);
    cudaStreamWaitEvent(c->stream, done, 0);
    cudaEventDestroy(done);
  }
  GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  const cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return set_cuda_error(c, e, "lane execution");
  if (rc) return rc;
  // device status of every lane; a lane that saw an error is re-armed
  int* st = (int*)pinned(c, 4096 + (size_t)n * 64);
  for (int i = 0; i < k; ++i) {
    gdb_lane& L = c->lanes[i];
    GDB_CUDA(c, cudaMemcpy(st, &L.dctx->status, 4 * sizeof(int), cudaMemcpyDeviceToHost));
    if (st[0] != 0) {
      const int status = st[0], where = st[2];
      GDB_CUDA(c, arm_device_ctx(c, L.dctx, L.flags, L.stream, 0));
      GDB_CUDA(c, cudaStreamSynchronize(L.stream));
      char buf[160];
      snprintf(buf, sizeof buf, "lane %d: device reported %s at site %d", i, gdb_status_string(status),
               where);
      return set_error(c, status, buf);
    }
  }
  stage = (unsigned long long*)pinned(c, 4096 + (size_t)n * 64) + 512;
  c->last = gdb_run_stats{};
  for (uint32_t i = 0; i < n; ++i) {
    if (*(int*)(stage + 8 * i + 4)) return set_error(c, GDB_ERR_CAPACITY, "queue overflow in a lane");
    c->last.edges_processed += stage[8 * i];
    c->last.supersteps += (uint32_t)stage[8 * i + 1];
    if (stats_out)
      for (int j = 0; j < 4; ++j) stats_out[4 * i + j] = stage[8 * i + j];
  }
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last.kernel_ms = ms;
  c->last.launches = n;
  c->last.launched = (uint32_t)std::max(1, fit / k);
  c->last.participating = c->last.launched;
  return GDB_OK;
}

// Pinned staging layout: [0, 3072) run statistics of the callers,
// [3072, 3584) participating count, [3584, 4096) device status.
int finish_run(gdb_ctx* c) {
  char* base = (char*)pinned(c, 4096);
  if (!base) return set_error(c, GDB_ERR_OOM, "pinned staging");
  int* h = (int*)(base + 3584);
  // status, abort, err_where of the device context
  GDB_CUDA(c, cudaMemcpyAsync(h, &c->dctx->status, 4 * sizeof(int), cudaMemcpyDeviceToHost,
                              c->stream));
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return set_cuda_error(c, e, "kernel execution");
  const int status = h[0], where = h[2];
  if (status != 0) {
    int skip = 0;
    cudaMemcpy(&skip, &c->dctx->skip, sizeof(int), cudaMemcpyDeviceToHost);
    reset_device_ctx(c, skip);
    char buf[160];
    snprintf(buf, sizeof buf, "device reported %s at site %d", gdb_status_string(status), where);
    c->err = buf;
    return status;
  }
  return GDB_OK;
}

int read_participating(gdb_ctx* c, int* n) {
  char* base = (char*)pinned(c, 4096);
  if (!base) return set_error(c, GDB_ERR_OOM, "pinned staging");
  int* h = (int*)(base + 3072);
  GDB_CUDA(c, cudaMemcpyAsync(h, &c->dctx->num_participating, sizeof(int), cudaMemcpyDeviceToHost,
                              c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  *n = h[0];
  return GDB_OK;
}

// Capacity of a frontier's chunk entries: sum of ceil(d / kChunk) over the
// heavy vertices, at most E / kChunk + nheavy.
uint32_t chunk_capacity(const gdb_graph* g) {
  return (uint32_t)std::max<uint64_t>(g->E / gdb::kChunk + g->nheavy + 1, 1);
}

bool graph_ok(gdb_ctx* c, gdb_graph* g) { return c && g && g->ctx == c; }

cudaError_t dev_alloc(gdb_ctx* c, void** p, size_t bytes) {
  return cudaMallocAsync(p, bytes, c->stream);
}

void dev_free(gdb_ctx* c, void* p) {
  if (p) cudaFreeAsync(p, c->stream);
}

}  // namespace gdbi

gdb::GraphView gdb_graph::view() const {
  gdb::GraphView v;
  v.V = V;
  v.E = (uint32_t)E;
  v.row = row;
  v.col = col;
  v.w = w;
  v.nheavy = nheavy;
  v.nheavy_chunks = nheavy_chunks;
  v.heavy_v = heavy_v;
  v.heavy_chunk = heavy_chunk;
  v.heavy_bits = heavy_bits;
  return v;
}

using namespace gdbi;

extern "C" {

int gdb_abi_version(void) { return GDB_ABI_VERSION; }

void gdb_options_default(gdb_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->device = -1;
  o->block_size = 512;
  o->max_ctas = 0;
  o->oversubscribe = 0;
  o->lock = GDB_LOCK_FREE;
  o->barrier = GDB_BARRIER_XF;
  o->schedule = GDB_SCHED_PLAIN;
  o->xf_release = gdb::kXfAuto;
  o->timeout_ns = 2000000000ull;
}

const char* gdb_status_string(int s) {
  switch (s) {
    case GDB_OK: return "GDB_OK";
    case GDB_ERR_INVALID: return "GDB_ERR_INVALID";
    case GDB_ERR_CUDA: return "GDB_ERR_CUDA";
    case GDB_ERR_OOM: return "GDB_ERR_OOM";
    case GDB_ERR_TIMEOUT: return "GDB_ERR_TIMEOUT";
    case GDB_ERR_CAPACITY: return "GDB_ERR_CAPACITY";
    case GDB_ERR_NOT_CORESIDENT: return "GDB_ERR_NOT_CORESIDENT";
    case GDB_ERR_UNSUPPORTED: return "GDB_ERR_UNSUPPORTED";
    default: return "GDB_ERR_UNKNOWN";
  }
}

static int check_options(const gdb_options* o) {
  if (o->block_size != 0 && (o->block_size < 64 || o->block_size > 1024 || (o->block_size & 31)))
    return GDB_ERR_INVALID;
  if (o->lock < GDB_LOCK_TICKET || o->lock > GDB_LOCK_FREE) return GDB_ERR_INVALID;
  if (o->barrier < GDB_BARRIER_XF || o->barrier > GDB_BARRIER_RELAUNCH_GRAPH) return GDB_ERR_INVALID;
  if (o->schedule < GDB_SCHED_PLAIN || o->schedule > GDB_SCHED_LEARNED) return GDB_ERR_INVALID;
  if (o->max_ctas < 0 || o->oversubscribe < 0) return GDB_ERR_INVALID;
  if (o->xf_release < 0 || o->xf_release > 4) return GDB_ERR_INVALID;
  if (o->sssp_split < -1 || o->sssp_split > 1) return GDB_ERR_INVALID;
  if (o->pull_bitmap_kb < -1 || o->pull_bitmap_kb > 64) return GDB_ERR_INVALID;
  return GDB_OK;
}

int gdb_ctx_create(const gdb_options* opt, gdb_ctx** out) {
  if (!out) return GDB_ERR_INVALID;
  *out = nullptr;
  gdb_options o;
  gdb_options_default(&o);
  if (opt) o = *opt;
  if (o.block_size == 0) o.block_size = 512;
  if (o.timeout_ns == 0) o.timeout_ns = 2000000000ull;
  if (check_options(&o) != GDB_OK) return GDB_ERR_INVALID;
  gdb_ctx* c = new gdb_ctx();
  c->opt = o;
  int dev = o.device;
  if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return GDB_ERR_CUDA;
  }
  c->device = dev;
  cudaDeviceProp prop;
  if (cudaSetDevice(dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return GDB_ERR_CUDA;
  }
  c->sm_count = prop.multiProcessorCount;
  c->cc_major = prop.major;
  c->cc_minor = prop.minor;
  c->total_mem = prop.totalGlobalMem;
  // at most 32 resident CTAs per SM on this architecture family
  c->flag_cap = std::max(64, c->sm_count * 32);
  // graphs, their partitions and per-call buffers come from the device's
  // stream-ordered pool; keep freed blocks cached in it (a graph created
  // and destroyed per request then costs no page mapping)
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  bool ok = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&c->ev0) == cudaSuccess && cudaEventCreate(&c->ev1) == cudaSuccess &&
            cudaMalloc(&c->dctx, sizeof(gdb::DeviceCtx)) == cudaSuccess &&
            cudaMalloc(&c->flags, (size_t)c->flag_cap * gdb::kLineInts * sizeof(int)) == cudaSuccess;
  if (!ok || reset_device_ctx(c, 0) != GDB_OK || bfs_prepare(c) != GDB_OK) {
    cudaGetLastError();
    gdb_ctx_destroy(c);
    return GDB_ERR_CUDA;
  }
  *out = c;
  return GDB_OK;
}

int gdb_ctx_destroy(gdb_ctx* c) {
  if (!c) return GDB_ERR_INVALID;
  if (c->stream) cudaStreamSynchronize(c->stream);
  lanes_destroy(c);
  if (c->ws) cudaFree(c->ws);
  if (c->pinned) cudaFreeHost(c->pinned);
  if (c->dctx) cudaFree(c->dctx);
  if (c->flags) cudaFree(c->flags);
  if (c->d_mlp) cudaFree(c->d_mlp);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  cudaGetLastError();
  delete c;
  return GDB_OK;
}

int gdb_ctx_set_options(gdb_ctx* c, const gdb_options* opt) {
  if (!c || !opt) return GDB_ERR_INVALID;
  gdb_options o = *opt;
  if (o.block_size == 0) o.block_size = 512;
  if (o.timeout_ns == 0) o.timeout_ns = 2000000000ull;
  if (check_options(&o) != GDB_OK) return GDB_ERR_INVALID;
  o.device = c->device;
  const bool mode_change = o.xf_release != c->opt.xf_release;
  c->opt = o;
  // per-slave flags read "arrived" as != 0: clear the epochs the broadcast
  // form leaves in them
  if (mode_change) return reset_device_ctx(c, 0);
  return GDB_OK;
}

int gdb_ctx_get_options(gdb_ctx* c, gdb_options* opt) {
  if (!c || !opt) return GDB_ERR_INVALID;
  *opt = c->opt;
  return GDB_OK;
}

int gdb_ctx_stream(gdb_ctx* c, void** s) {
  if (!c || !s) return GDB_ERR_INVALID;
  *s = (void*)c->stream;
  return GDB_OK;
}

const char* gdb_last_error(gdb_ctx* c) { return c ? c->err.c_str() : "null context"; }

int gdb_last_run_stats(gdb_ctx* c, gdb_run_stats* s) {
  if (!c || !s) return GDB_ERR_INVALID;
  *s = c->last;
  return GDB_OK;
}

int gdb_debug_stall_master(gdb_ctx* c, int after) {
  if (!c) return GDB_ERR_INVALID;
  c->stall_after = after < 0 ? -1 : after;
  GDB_CUDA(c, cudaMemcpyAsync(&c->dctx->stall_after, &c->stall_after, sizeof(int),
                              cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  return GDB_OK;
}

static int graph_common(gdb_ctx* c, uint32_t V, uint64_t E) {
  if (!c) return GDB_ERR_INVALID;
  if (V == 0 || V >= 0x7fffffffu || E >= 0xffffffffull) {
    return set_error(c, GDB_ERR_INVALID, "graph needs 0 < V < 2^31 and E < 2^32");
  }
  return GDB_OK;
}

int gdb_graph_create(gdb_ctx* c, uint32_t V, uint64_t E, const uint32_t* row, const uint32_t* col,
                     const uint32_t* w, gdb_graph** out) {
  if (!out || !row || (E && !col)) return GDB_ERR_INVALID;
  *out = nullptr;
  int rc = graph_common(c, V, E);
  if (rc) return rc;
  if (row[0] != 0 || row[V] != E) return set_error(c, GDB_ERR_INVALID, "row_ptr[0] != 0 or row_ptr[V] != E");
  gdb_graph* g = new gdb_graph();
  g->ctx = c;
  g->V = V;
  g->E = E;
  const size_t eb = std::max<uint64_t>(E, 1) * 4;
  cudaError_t e = dev_alloc(c, (void**)&g->row, (size_t)(V + 1) * 4);
  if (e == cudaSuccess) e = dev_alloc(c, (void**)&g->col, eb);
  if (e == cudaSuccess && w) e = dev_alloc(c, (void**)&g->w, eb);
  if (e == cudaSuccess) e = cudaMemcpyAsync(g->row, row, (size_t)(V + 1) * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && E) e = cudaMemcpyAsync(g->col, col, E * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && w && E) e = cudaMemcpyAsync(g->w, w, E * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    rc = set_cuda_error(c, e, "graph upload");
    gdb_graph_destroy(g);
    return rc;
  }
  rc = build_heavy_table(g);
  if (rc) {
    gdb_graph_destroy(g);
    return rc;
  }
  *out = g;
  return GDB_OK;
}

int gdb_graph_create_device(gdb_ctx* c, uint32_t V, uint64_t E, const uint32_t* d_row,
                            const uint32_t* d_col, const uint32_t* d_w, gdb_graph** out) {
  if (!out || !d_row || (E && !d_col)) return GDB_ERR_INVALID;
  *out = nullptr;
  int rc = graph_common(c, V, E);
  if (rc) return rc;
  uint32_t ends[2] = {1, 0};
  cudaError_t e = cudaMemcpy(&ends[0], d_row, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&ends[1], d_row + V, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_cuda_error(c, e, "row_ptr read-back");
  if (ends[0] != 0 || ends[1] != E) return set_error(c, GDB_ERR_INVALID, "row_ptr[0] != 0 or row_ptr[V] != E");
  gdb_graph* g = new gdb_graph();
  g->ctx = c;
  g->V = V;
  g->E = E;
  g->row = const_cast<uint32_t*>(d_row);
  g->col = const_cast<uint32_t*>(d_col);
  g->w = const_cast<uint32_t*>(d_w);
  g->owns = false;
  g->owns_w = false;
  rc = build_heavy_table(g);
  if (rc) {
    gdb_graph_destroy(g);
    return rc;
  }
  *out = g;
  return GDB_OK;
}

int gdb_graph_set_weights(gdb_graph* g, const uint32_t* w) {
  if (!g || !w) return GDB_ERR_INVALID;
  gdb_ctx* c = g->ctx;
  if (!g->w || !g->owns_w) {
    g->w = nullptr;
    GDB_CUDA(c, dev_alloc(c, (void**)&g->w, std::max<uint64_t>(g->E, 1) * 4));
    g->owns_w = true;
  }
  g->wmean = -1.0;
  arc_split_drop(g);
  if (g->E) GDB_CUDA(c, cudaMemcpyAsync(g->w, w, g->E * 4, cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  return GDB_OK;
}

int gdb_graph_set_symmetric(gdb_graph* g, int symmetric) {
  if (!g || (symmetric != 0 && symmetric != 1)) return GDB_ERR_INVALID;
  if ((bool)symmetric != g->symmetric) {
    cudaStreamSynchronize(g->ctx->stream);
    arc_split_drop(g);  // the partition's transposed half depends on it
    g->symmetric = symmetric != 0;
  }
  return GDB_OK;
}

int gdb_graph_destroy(gdb_graph* g) {
  if (!g) return GDB_ERR_INVALID;
  gdb_ctx* c = g->ctx;
  // work on any stream may still read the graph (batches, server slots)
  cudaDeviceSynchronize();
  arc_split_drop(g);
  if (g->owns) {
    dev_free(c, g->row);
    dev_free(c, g->col);
  }
  if (g->owns_w) dev_free(c, g->w);
  dev_free(c, g->heavy_v);
  dev_free(c, g->heavy_chunk);
  dev_free(c, g->heavy_bits);
  cudaGetLastError();
  delete g;
  return GDB_OK;
}

int gdb_graph_info(gdb_graph* g, uint32_t* V, uint64_t* E, uint32_t* heavy) {
  if (!g) return GDB_ERR_INVALID;
  if (V) *V = g->V;
  if (E) *E = g->E;
  if (heavy) *heavy = g->nheavy;
  return GDB_OK;
}

int gdb_device_info_get(gdb_ctx* c, gdb_device_info* info) {
  if (!c || !info) return GDB_ERR_INVALID;
  info->device = c->device;
  info->sm_count = c->sm_count;
  info->cc_major = c->cc_major;
  info->cc_minor = c->cc_minor;
  info->total_mem = c->total_mem;
  info->flag_capacity = c->flag_cap;
  info->occupancy_per_sm = gdbi::traversal_occupancy(c, c->opt.block_size);
  return GDB_OK;
}

}  // extern "C"
