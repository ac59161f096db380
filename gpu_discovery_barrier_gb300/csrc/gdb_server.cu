// Request loop with continuous batching over graphs resident in HBM.
//
// A dispatcher thread owns every CUDA call of the server.  Each pass it
//  1. retires finished slots (an event per launch): reads the device
//     status, copies the result from the slot's pinned staging into the
//     caller's buffer, frees the request's pool block;
//  2. admits queued requests in arrival order, bypassing ones whose
//     footprint does not fit yet, while a slot and a first-fit pool block
//     are free: source upload, persistent launch, status and result
//     read-back and a completion event, all enqueued on the slot's stream.
// Slots have their own discovery context and barrier flags, so launches on
// different slots overlap on the device; each launch is capped at a share
// of the co-resident CTAs (options.max_ctas, default occupancy x SMs /
// slots), which keeps room on the GPU for the other slots' launches.  The
// discovery protocol keeps every launch correct whatever share of the GPU
// it actually gets: only CTAs that are running when the poll closes take
// part in its barriers.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gdb_internal.h"

using namespace gdbi;

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

constexpr size_t kAlign = 256;
size_t round_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

struct Slot {
  gdb::DeviceCtx* dctx = nullptr;
  int* flags = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  char* pin = nullptr;        // [0, 16) status, [16, 20) source, [64, 68) overflow, [256, ...) staging
  size_t pin_bytes = 0;
  int64_t req = -1;
};

struct Req {
  uint64_t id = 0;
  uint32_t graph = 0, app = 0, src = 0;
  void* out = nullptr;
  Clock::time_point t_submit, t_admit;
  size_t off = 0, bytes = 0, ws_bytes = 0;
  int slot = -1;
  gdb_request_info info{};
};

struct GraphEntry {
  gdb_graph* g = nullptr;
  uint32_t delta = 0;  // SSSP bucket width under the server's schedule
  uint32_t light = GDB_LONESTAR_INF;  // and its light-arc bound
};

}  // namespace

struct gdb_server {
  gdb_ctx* user = nullptr;
  gdb_ctx* sc = nullptr;  // launch parameters (options, selector); its stream is unused
  std::vector<GraphEntry> graphs;
  std::vector<Slot> slots;
  char* pool = nullptr;
  size_t pool_bytes = 0;
  std::map<size_t, size_t> free_blocks;  // offset -> length
  std::deque<uint64_t> pending;
  std::unordered_map<uint64_t, Req> reqs;
  std::deque<gdb_request_info> completed;
  uint64_t next_id = 1;
  size_t outstanding = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread th;
  bool stop = false;
  int fatal = GDB_OK;
};

namespace {

bool pool_alloc(gdb_server* s, size_t bytes, size_t* off) {
  for (auto it = s->free_blocks.begin(); it != s->free_blocks.end(); ++it) {
    if (it->second < bytes) continue;
    *off = it->first;
    const size_t rest = it->second - bytes;
    const size_t roff = it->first + bytes;
    s->free_blocks.erase(it);
    if (rest) s->free_blocks[roff] = rest;
    return true;
  }
  return false;
}

void pool_free(gdb_server* s, size_t off, size_t bytes) {
  auto it = s->free_blocks.emplace(off, bytes).first;
  auto nx = std::next(it);
  if (nx != s->free_blocks.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    s->free_blocks.erase(nx);
  }
  if (it != s->free_blocks.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      s->free_blocks.erase(it);
    }
  }
}

int slot_arm(gdb_server* s, Slot& sl) {
  gdb::DeviceCtx h;
  std::memset(&h, 0, sizeof(h));
  h.poll_open = 1;
  h.stall_after = -1;
  cudaError_t e = cudaMemcpyAsync(sl.dctx, &h, sizeof(h), cudaMemcpyHostToDevice, sl.stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(sl.flags, 0, (size_t)s->sc->flag_cap * gdb::kLineInts * sizeof(int), sl.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(sl.stream);
  return e == cudaSuccess ? GDB_OK : GDB_ERR_CUDA;
}

size_t app_workspace(const gdb_graph* g, uint32_t app) {
  switch (app) {
    case GDB_APP_BFS: return bfs_workspace_bytes(g);
    case GDB_APP_SSSP: return sssp_workspace_bytes(g);
    default: return bc_workspace_bytes(g);
  }
}

// Pool block: [result V x 4][source][app workspace].
size_t footprint(const gdb_graph* g, uint32_t app) {
  return round_up((size_t)g->V * 4) + kAlign + round_up(app_workspace(g, app));
}

void complete(gdb_server* s, Req& r, int status, double run_ms) {
  r.info.status = status;
  r.info.run_ms = run_ms;
  r.info.total_ms = ms_since(r.t_submit, Clock::now());
  s->completed.push_back(r.info);
  s->reqs.erase(r.id);
  --s->outstanding;
  s->cv_done.notify_all();
}

int launch(gdb_server* s, Slot& sl, Req& r) {
  gdb_ctx* c = s->sc;
  const GraphEntry& ge = s->graphs[r.graph];
  gdb_graph* g = ge.g;
  const size_t vb = (size_t)g->V * 4;
  if (sl.pin_bytes < 256 + vb) {
    if (sl.pin) cudaFreeHost(sl.pin);
    sl.pin = nullptr;
    sl.pin_bytes = 0;
    GDB_CUDA(c, cudaHostAlloc((void**)&sl.pin, 256 + vb, cudaHostAllocDefault));
    sl.pin_bytes = 256 + vb;
  }
  char* base = s->pool + r.off;
  char* out = base;
  uint32_t* d_src = (uint32_t*)(base + round_up(vb));
  char* ws = base + round_up(vb) + kAlign;
  *(uint32_t*)(sl.pin + 16) = r.src;
  GDB_CUDA(c, cudaMemcpyAsync(d_src, sl.pin + 16, 4, cudaMemcpyHostToDevice, sl.stream));
  gdb::DiscoveryArgs proto;
  proto.ctx = sl.dctx;
  proto.flags = sl.flags;
  proto.flag_capacity = c->flag_cap;
  proto.lock_kind = c->opt.lock;
  proto.expected = 0;
  proto.timeout_ns = c->opt.timeout_ns ? c->opt.timeout_ns : 2000000000ull;
  proto.close_wait_ns = 50000ull;
  proto.launch_id = 1;
  proto.xf_release = gdb::kXfAuto;
  GDB_CUDA(c, cudaEventRecord(sl.ev0, sl.stream));
  int rc;
  if (r.app == GDB_APP_BFS)
    rc = bfs_enqueue(c, g, ws, d_src, 1, (uint32_t*)out, sl.stream, proto, false);
  else if (r.app == GDB_APP_SSSP)
    rc = sssp_enqueue(c, g, ws, d_src, 1, (uint32_t*)out, sl.stream, proto, ge.delta, ge.light);
  else
    rc = bc_enqueue(c, g, ws, d_src, 1, (float*)out, sl.stream, proto);
  if (rc) return rc;
  // the workspace's counter block is its last 512 bytes; its overflow word at +160
  GDB_CUDA(c, cudaMemcpyAsync(sl.pin, &sl.dctx->status, 16, cudaMemcpyDeviceToHost, sl.stream));
  GDB_CUDA(c, cudaMemcpyAsync(sl.pin + 64, ws + r.ws_bytes - 512 + 160, 4, cudaMemcpyDeviceToHost,
                              sl.stream));
  GDB_CUDA(c, cudaMemcpyAsync(sl.pin + 256, out, vb, cudaMemcpyDeviceToHost, sl.stream));
  GDB_CUDA(c, cudaEventRecord(sl.ev1, sl.stream));
  return GDB_OK;
}

void retire(gdb_server* s, int si, cudaError_t q) {
  Slot& sl = s->slots[si];
  Req& r = s->reqs[(uint64_t)sl.req];
  int status = GDB_OK;
  float ms = 0.f;
  if (q != cudaSuccess) {
    status = GDB_ERR_CUDA;
    s->fatal = GDB_ERR_CUDA;
  } else {
    status = *(int*)sl.pin;
    if (status != GDB_OK) slot_arm(s, sl);
    else if (*(int*)(sl.pin + 64)) status = GDB_ERR_CAPACITY;
    cudaEventElapsedTime(&ms, sl.ev0, sl.ev1);
    if (status == GDB_OK) std::memcpy(r.out, sl.pin + 256, (size_t)s->graphs[r.graph].g->V * 4);
  }
  pool_free(s, r.off, r.bytes);
  sl.req = -1;
  complete(s, r, status, ms);
}

void dispatcher(gdb_server* s) {
  cudaSetDevice(s->sc->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    bool progressed = false, busy = false;
    for (int i = 0; i < (int)s->slots.size(); ++i) {
      Slot& sl = s->slots[i];
      if (sl.req < 0) continue;
      const cudaError_t q = cudaEventQuery(sl.ev1);
      if (q == cudaErrorNotReady) {
        busy = true;
        continue;
      }
      retire(s, i, q);
      progressed = true;
    }
    for (auto it = s->pending.begin(); it != s->pending.end() && s->fatal == GDB_OK;) {
      int free_slot = -1;
      for (int i = 0; i < (int)s->slots.size(); ++i)
        if (s->slots[i].req < 0) {
          free_slot = i;
          break;
        }
      if (free_slot < 0) break;
      Req& r = s->reqs[*it];
      size_t off = 0;
      if (!pool_alloc(s, r.bytes, &off)) {
        ++it;
        continue;
      }
      r.off = off;
      r.slot = free_slot;
      r.t_admit = Clock::now();
      r.info.queue_ms = ms_since(r.t_submit, r.t_admit);
      r.info.slot = (uint32_t)free_slot;
      Slot& sl = s->slots[free_slot];
      sl.req = (int64_t)r.id;
      it = s->pending.erase(it);
      progressed = true;
      const int rc = launch(s, sl, r);
      if (rc != GDB_OK) {
        // nothing of the request may still run: wait for its stream, then fail it
        cudaStreamSynchronize(sl.stream);
        cudaGetLastError();
        slot_arm(s, sl);
        pool_free(s, r.off, r.bytes);
        sl.req = -1;
        complete(s, r, rc, 0.0);
      } else {
        busy = true;
      }
    }
    if (s->fatal != GDB_OK) {
      // a sticky CUDA error: fail everything still queued
      while (!s->pending.empty()) {
        Req& r = s->reqs[s->pending.front()];
        s->pending.pop_front();
        complete(s, r, s->fatal, 0.0);
      }
    }
    if (s->stop && s->pending.empty() && !busy) break;
    if (!busy && (s->pending.empty() || s->fatal != GDB_OK)) {
      s->cv_work.wait(lk);
      continue;
    }
    if (!progressed) {
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      lk.lock();
    }
  }
}

}  // namespace

extern "C" {

int gdb_server_create(gdb_ctx* c, uint32_t slots, uint64_t pool_bytes, gdb_server** out) {
  if (!c || !out) return GDB_ERR_INVALID;
  *out = nullptr;
  if (slots == 0) slots = 8;
  if (pool_bytes == 0) pool_bytes = 1ull << 30;
  if (slots > 64) return set_error(c, GDB_ERR_INVALID, "at most 64 slots");
  gdb_options o = c->opt;
  o.barrier = GDB_BARRIER_XF;
  if (o.max_ctas == 0) {
    const int occ = gdbi::traversal_occupancy(c, o.block_size);
    if (occ <= 0) return set_error(c, GDB_ERR_INVALID, "traversal kernels do not fit at this block size");
    o.max_ctas = std::max(1, occ * c->sm_count / (int)slots);
  }
  gdb_server* s = new gdb_server();
  s->user = c;
  int rc = gdb_ctx_create(&o, &s->sc);
  if (rc) {
    delete s;
    return rc;
  }
  if (!c->h_mlp.empty()) gdb_selector_set(s->sc, c->h_mlp.data());
  cudaError_t e = cudaMalloc((void**)&s->pool, pool_bytes);
  if (e != cudaSuccess) {
    gdb_ctx_destroy(s->sc);
    delete s;
    return set_error(c, GDB_ERR_OOM, "server pool");
  }
  s->pool_bytes = pool_bytes;
  s->free_blocks[0] = pool_bytes;
  s->slots.resize(slots);
  for (auto& sl : s->slots) {
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.ev1);
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl.dctx, sizeof(gdb::DeviceCtx));
    if (e == cudaSuccess)
      e = cudaMalloc((void**)&sl.flags, (size_t)s->sc->flag_cap * gdb::kLineInts * sizeof(int));
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&sl.pin, 4096, cudaHostAllocDefault);
    if (e == cudaSuccess) sl.pin_bytes = 4096;
    if (e == cudaSuccess && slot_arm(s, sl) != GDB_OK) e = cudaErrorUnknown;
  }
  if (e != cudaSuccess) {
    gdb_server_destroy(s);
    return set_cuda_error(c, e, "server slots");
  }
  s->th = std::thread(dispatcher, s);
  *out = s;
  return GDB_OK;
}

int gdb_server_add_graph(gdb_server* s, gdb_graph* g, uint32_t* graph_id) {
  if (!s || !g || g->ctx != s->user || !graph_id) return GDB_ERR_INVALID;
  GraphEntry ge;
  ge.g = g;
  if (g->w) {
    bool relaunch = false;
    int rc = sssp_plan(s->sc, g, 1, false, &ge.delta, &relaunch, &ge.light);
    if (rc) return rc;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  // staging for the result read-back of every idle slot (busy ones grow
  // theirs at their next launch)
  const size_t need = 256 + (size_t)g->V * 4;
  for (auto& sl : s->slots) {
    if (sl.req >= 0 || sl.pin_bytes >= need) continue;
    if (sl.pin) cudaFreeHost(sl.pin);
    sl.pin = nullptr;
    sl.pin_bytes = 0;
    if (cudaHostAlloc((void**)&sl.pin, need, cudaHostAllocDefault) != cudaSuccess)
      return set_error(s->user, GDB_ERR_OOM, "server staging");
    sl.pin_bytes = need;
  }
  *graph_id = (uint32_t)s->graphs.size();
  s->graphs.push_back(ge);
  return GDB_OK;
}

int gdb_server_submit(gdb_server* s, uint32_t graph_id, uint32_t app, uint32_t src, void* out,
                      uint64_t* request_id) {
  if (!s || !out || app < GDB_APP_BFS || app > GDB_APP_BC) return GDB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (graph_id >= s->graphs.size()) return GDB_ERR_INVALID;
  gdb_graph* g = s->graphs[graph_id].g;
  if (src >= g->V) return GDB_ERR_INVALID;
  if (app == GDB_APP_SSSP && !g->w) return GDB_ERR_INVALID;
  if (s->fatal != GDB_OK) return s->fatal;
  Req r;
  r.id = s->next_id++;
  r.graph = graph_id;
  r.app = app;
  r.src = src;
  r.out = out;
  r.t_submit = Clock::now();
  r.ws_bytes = app_workspace(g, app);
  r.bytes = footprint(g, app);
  if (r.bytes > s->pool_bytes) return GDB_ERR_CAPACITY;
  r.info.id = r.id;
  r.info.app = app;
  r.info.graph = graph_id;
  r.info.src = src;
  r.info.footprint = r.bytes;
  s->reqs.emplace(r.id, r);
  s->pending.push_back(r.id);
  ++s->outstanding;
  if (request_id) *request_id = r.id;
  s->cv_work.notify_one();
  return GDB_OK;
}

int gdb_server_poll(gdb_server* s, gdb_request_info* info, uint32_t max, uint32_t* n) {
  if (!s || !n || (max && !info)) return GDB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  uint32_t k = 0;
  while (k < max && !s->completed.empty()) {
    info[k++] = s->completed.front();
    s->completed.pop_front();
  }
  *n = k;
  return GDB_OK;
}

int gdb_server_drain(gdb_server* s, double timeout_s) {
  if (!s) return GDB_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto done = [&] { return s->outstanding == 0; };
  if (timeout_s <= 0) {
    s->cv_done.wait(lk, done);
  } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return GDB_ERR_TIMEOUT;
  }
  return s->fatal;
}

int gdb_server_destroy(gdb_server* s) {
  if (!s) return GDB_OK;
  if (s->th.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
      s->cv_work.notify_all();
    }
    s->th.join();
  }
  for (auto& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.ev0) cudaEventDestroy(sl.ev0);
    if (sl.ev1) cudaEventDestroy(sl.ev1);
    if (sl.dctx) cudaFree(sl.dctx);
    if (sl.flags) cudaFree(sl.flags);
    if (sl.pin) cudaFreeHost(sl.pin);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  if (s->pool) cudaFree(s->pool);
  if (s->sc) gdb_ctx_destroy(s->sc);
  cudaGetLastError();
  delete s;
  return GDB_OK;
}

}  // extern "C"
