// Discovery protocol and barrier entry points: context (re)initialisation,
// protocol timing, occupancy test and the barrier latency benchmark.
//
// Kernels mirror the reference's occupancy_test.cl (run_prot, run_test) and
// add the barrier microbenchmark: XF over discovered CTAs, XF over a fixed
// grid at the API occupancy (gbar_cl.h), cooperative_groups grid.sync and
// per-superstep relaunch (plain and as a replayed CUDA graph).
#include <algorithm>

#include "gdb_internal.h"

namespace {

using gdb::DiscoveryArgs;
using gdb::LocalCtx;

// run_prot (occupancy_tests/src/kernels/occupancy_test.cl:13-15)
__global__ void k_run_prot(DiscoveryArgs a) {
  __shared__ LocalCtx l;
  gdb::discover(a, &l);
}

// run_test (occupancy_test.cl:8-12): protocol followed by one barrier.
__global__ void k_run_test(DiscoveryArgs a) {
  __shared__ LocalCtx l;
  extern __shared__ int lms[];
  if (!gdb::discover(a, &l)) return;
  if (threadIdx.x == 0 && blockDim.x > 1) lms[0] = l.id;  // touch the dynamic allocation
  gdb::xf_barrier(a, &l);
  gdb::xf_finish(a, &l);
}

// `iters` empty supersteps; participant 0 times barriers 2..iters+1 with
// %globaltimer so launch and discovery are excluded.
__global__ void k_bench_xf(DiscoveryArgs a, int iters, unsigned long long* out_ns) {
  __shared__ LocalCtx l;
  if (!gdb::discover(a, &l)) return;
  if (!gdb::xf_barrier(a, &l)) return;
  unsigned long long t0 = gdb::globaltimer();
  for (int i = 0; i < iters; ++i)
    if (!gdb::xf_barrier(a, &l)) return;
  if (l.id == 0 && threadIdx.x == 0) {
    out_ns[0] = gdb::globaltimer() - t0;
    out_ns[1] = (unsigned long long)l.P;
  }
  gdb::xf_finish(a, &l);
}

__global__ void k_bench_grid(int iters, unsigned long long* out_ns) {
  auto grid = cooperative_groups::this_grid();
  grid.sync();
  unsigned long long t0 = gdb::globaltimer();
  for (int i = 0; i < iters; ++i) grid.sync();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    out_ns[0] = gdb::globaltimer() - t0;
    out_ns[1] = (unsigned long long)gridDim.x;
  }
}

// One superstep of the relaunch baseline: read and update a word so the
// launches are not empty.
__global__ void k_bench_step(unsigned long long* counter) {
  if (blockIdx.x == 0 && threadIdx.x == 0) counter[2] += 1;
}

}  // namespace

using namespace gdbi;

extern "C" {

int gdb_init_discovery_kernel_ctx(gdb_ctx* c) {
  if (!c) return GDB_ERR_INVALID;
  return reset_device_ctx(c, 0);
}

int gdb_init_discovery_kernel_ctx_skip(gdb_ctx* c, int skip) {
  if (!c) return GDB_ERR_INVALID;
  return reset_device_ctx(c, skip ? 1 : 0);
}

int gdb_number_of_participating_groups(gdb_ctx* c) {
  if (!c) return GDB_ERR_INVALID;
  int n = 0;
  int rc = read_participating(c, &n);
  return rc ? rc : n;
}

static int read_skip(gdb_ctx* c, int* skip) {
  GDB_CUDA(c, cudaMemcpy(skip, &c->dctx->skip, sizeof(int), cudaMemcpyDeviceToHost));
  return GDB_OK;
}

int gdb_api_occupancy(gdb_ctx* c, int wgs, int lms, int* ctas) {
  if (!c || !ctas || wgs <= 0 || wgs > 1024 || lms < 0) return GDB_ERR_INVALID;
  int occ = 0;
  GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_run_test, wgs, lms));
  *ctas = occ * c->sm_count;
  return GDB_OK;
}

int gdb_time_protocol(gdb_ctx* c, int upper_bound, int wgs, double* ns) {
  if (!c || !ns || upper_bound <= 0 || wgs <= 0 || wgs > 1024) return GDB_ERR_INVALID;
  int skip = 0;
  int rc = read_skip(c, &skip);
  if (rc) return rc;
  // init_discovery_kernel_ctx before the timed launch (discovery.h:74)
  rc = reset_device_ctx(c, skip);
  if (rc) return rc;
  Shape s;
  s.grid = upper_bound;
  s.block = wgs;
  int occ = 0;
  GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_run_prot, wgs, 0));
  s.occ_per_sm = occ;
  s.fit = occ * c->sm_count;
  DiscoveryArgs a = discovery_args(c, s);
  GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  k_run_prot<<<upper_bound, wgs, 0, c->stream>>>(a);
  GDB_CUDA(c, cudaGetLastError());
  GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  rc = finish_run(c);
  if (rc) return rc;
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  *ns = (double)ms * 1e6;
  c->last = gdb_run_stats{};
  c->last.launched = upper_bound;
  c->last.launches = 1;
  c->last.kernel_ms = ms;
  int n = 0;
  rc = read_participating(c, &n);
  c->last.participating = n;
  return rc;
}

int gdb_occupancy_test(gdb_ctx* c, int wgc, int wgs, int lms, int* participating) {
  if (!c || !participating || wgc <= 0 || wgs <= 0 || wgs > 1024 || lms < 0) return GDB_ERR_INVALID;
  int skip = 0;
  int rc = read_skip(c, &skip);
  if (rc) return rc;
  int occ = 0;
  GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_run_test, wgs, lms));
  if (occ <= 0) return set_error(c, GDB_ERR_INVALID, "run_test does not fit at this size");
  const int fit = occ * c->sm_count;
  // With skip every launched CTA must be co-resident for the barrier to
  // finish; that is only guaranteed up to the API occupancy.
  if (skip && wgc > fit)
    return set_error(c, GDB_ERR_NOT_CORESIDENT, "skip=1 launch above the API occupancy");
  if (lms > 48 * 1024)
    GDB_CUDA(c, cudaFuncSetAttribute(k_run_test, cudaFuncAttributeMaxDynamicSharedMemorySize, lms));
  Shape s;
  s.grid = wgc;
  s.block = wgs;
  s.occ_per_sm = occ;
  s.fit = fit;
  DiscoveryArgs a = discovery_args(c, s);
  GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  k_run_test<<<wgc, wgs, lms, c->stream>>>(a);
  GDB_CUDA(c, cudaGetLastError());
  GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  rc = finish_run(c);
  if (rc) return rc;
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last = gdb_run_stats{};
  c->last.launched = wgc;
  c->last.launches = 1;
  c->last.kernel_ms = ms;
  int n = 0;
  rc = read_participating(c, &n);
  c->last.participating = n;
  *participating = n;
  return rc;
}

int gdb_barrier_bench(gdb_ctx* c, int kind, int wgs, int iters, double* ns_per, int* groups) {
  if (!c || !ns_per || iters <= 0) return GDB_ERR_INVALID;
  if (wgs == 0) wgs = c->opt.block_size;
  if (wgs < 32 || wgs > 1024) return GDB_ERR_INVALID;
  unsigned long long* d = (unsigned long long*)workspace(c, 64);
  if (!d) return GDB_ERR_OOM;
  GDB_CUDA(c, cudaMemsetAsync(d, 0, 64, c->stream));
  unsigned long long* h = (unsigned long long*)pinned(c, 64);
  if (!h) return GDB_ERR_OOM;
  int rc = GDB_OK;
  c->last = gdb_run_stats{};
  if (kind == GDB_BARRIER_XF || kind == GDB_BARRIER_XF_FIXED) {
    Shape s;
    rc = persistent_shape(c, (const void*)k_bench_xf, wgs, 0, &s, kind == GDB_BARRIER_XF);
    if (rc) return rc;
    if (kind == GDB_BARRIER_XF_FIXED) {
      s.grid = std::min(s.grid, s.fit);
      rc = reset_device_ctx(c, 1);
    } else {
      rc = reset_device_ctx(c, 0);
    }
    if (rc) return rc;
    DiscoveryArgs a = discovery_args(c, s);
    k_bench_xf<<<s.grid, wgs, 0, c->stream>>>(a, iters, d);
    GDB_CUDA(c, cudaGetLastError());
    rc = finish_run(c);
    if (kind == GDB_BARRIER_XF_FIXED) reset_device_ctx(c, 0);
    if (rc) return rc;
    GDB_CUDA(c, cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost));
    *ns_per = (double)h[0] / iters;
    if (groups) *groups = (int)h[1];
    c->last.launched = s.grid;
    c->last.participating = (uint32_t)h[1];
    c->last.supersteps = iters;
    c->last.launches = 1;
    return GDB_OK;
  }
  if (kind == GDB_BARRIER_GRID_SYNC) {
    int occ = 0;
    GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bench_grid, wgs, 0));
    int grid = occ * c->sm_count;
    if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
    void* args[] = {(void*)&iters, (void*)&d};
    GDB_CUDA(c, cudaLaunchCooperativeKernel((const void*)k_bench_grid, grid, wgs, args, 0, c->stream));
    GDB_CUDA(c, cudaStreamSynchronize(c->stream));
    GDB_CUDA(c, cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost));
    *ns_per = (double)h[0] / iters;
    if (groups) *groups = (int)h[1];
    c->last.launched = grid;
    c->last.participating = grid;
    c->last.supersteps = iters;
    c->last.launches = 1;
    return GDB_OK;
  }
  if (kind == GDB_BARRIER_RELAUNCH || kind == GDB_BARRIER_RELAUNCH_GRAPH) {
    int occ = 0;
    GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bench_step, wgs, 0));
    int grid = occ * c->sm_count;
    if (c->opt.max_ctas > 0) grid = std::min(grid, c->opt.max_ctas);
    // warm-up
    k_bench_step<<<grid, wgs, 0, c->stream>>>(d);
    GDB_CUDA(c, cudaGetLastError());
    float ms = 0;
    if (kind == GDB_BARRIER_RELAUNCH) {
      GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
      for (int i = 0; i < iters; ++i) k_bench_step<<<grid, wgs, 0, c->stream>>>(d);
      GDB_CUDA(c, cudaGetLastError());
      GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
      GDB_CUDA(c, cudaEventSynchronize(c->ev1));
      GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    } else {
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      GDB_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      for (int i = 0; i < iters; ++i) k_bench_step<<<grid, wgs, 0, c->stream>>>(d);
      cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
      if (e != cudaSuccess) return set_cuda_error(c, e, "graph capture");
      e = cudaGraphInstantiate(&exec, graph, 0);
      if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->stream);  // upload + warm
      if (e == cudaSuccess) e = cudaEventRecord(c->ev0, c->stream);
      if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->stream);
      if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      if (e != cudaSuccess) return set_cuda_error(c, e, "graph relaunch");
    }
    *ns_per = (double)ms * 1e6 / iters;
    if (groups) *groups = grid;
    c->last.launched = grid;
    c->last.participating = grid;
    c->last.supersteps = iters;
    c->last.launches = iters;
    c->last.kernel_ms = ms;
    return GDB_OK;
  }
  return GDB_ERR_INVALID;
}

}  // extern "C"
