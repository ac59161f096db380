// Relaunch forms of the persistent apps: one launch per superstep.
//
// The reference's multi-kernel apps run each superstep as its own kernel
// and read a stop flag back after it (pannotia/graph_app/sssp/sssp.cpp:290-344,
// mis/mis.cpp:314-364, color/color.cpp:294-334, bc/bc.cpp:322-420).  Here a
// step kernel runs exactly the superstep code of the persistent kernel;
// the loop state the persistent kernel keeps in registers lives in a
// control block instead.  Every CTA reads the block at the start of a
// launch, and the launch's last CTA to finish (a count-down over the grid)
// writes the next superstep's state -- all CTAs of a launch derive the same
// values, so the last one's are everybody's.
//
// Two drivers: GDB_BARRIER_RELAUNCH -- a host loop that reads the stop word
// back after every launch (the reference's pattern); GDB_BARRIER_RELAUNCH_GRAPH
// -- the step kernel as the body of a CUDA-graph WHILE node, whose
// condition the last CTA sets.  Both stop after `cap` launches at most
// (the app's bound on its supersteps), so neither can loop forever.
#pragma once

#include "gdb_internal.h"

namespace gdb {

struct StepCtl {
  uint32_t done;            // CTAs of the current launch that finished
  uint32_t stop;            // 1: the run is over
  uint32_t graph;           // 1: the step is the body of a WHILE node
  uint32_t capped;          // 1: stopped by the launch cap
  unsigned long long steps; // launches so far
  unsigned long long cap;   // launch cap
  uint32_t s[16];           // app state (32-bit)
  unsigned long long d[4];  // app state (64-bit)
};

// The app state at the start of this launch, in shared memory (thread 0
// loads it; every thread of the CTA calls this).
__device__ __forceinline__ const StepCtl& step_state(const StepCtl* ctl) {
  __shared__ StepCtl s;
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(ctl);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&s);
    for (unsigned i = 0; i < sizeof(StepCtl) / 4; ++i) dst[i] = __ldcg(src + i);
  }
  __syncthreads();
  return s;
}

// End of a step launch: the last CTA to finish calls next(state) in its
// thread 0 with every CTA's writes visible; next updates the state and
// returns whether another superstep follows.  Every thread calls this.
template <class Next>
__device__ __forceinline__ void step_end(StepCtl* ctl, cudaGraphConditionalHandle cond, Next&& next) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&ctl->done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  StepCtl st;
  uint32_t* dst = reinterpret_cast<uint32_t*>(&st);
  for (unsigned i = 0; i < sizeof(StepCtl) / 4; ++i) dst[i] = __ldcg(reinterpret_cast<uint32_t*>(ctl) + i);
  st.done = 0;
  ++st.steps;
  bool more = next(st);
  if (more && st.steps >= st.cap) {
    more = false;
    st.capped = 1;
  }
  st.stop = more ? 0u : 1u;
  for (unsigned i = 0; i < sizeof(StepCtl) / 4; ++i) reinterpret_cast<uint32_t*>(ctl)[i] = dst[i];
  __threadfence();
  if (st.graph) cudaGraphSetConditional(cond, more ? 1u : 0u);
}

}  // namespace gdb

namespace gdbi {

// Run init<<<grid, block>>>(args...) once, then step<<<grid, block>>>(args...,
// ctl, cond) until the step kernels set ctl->stop: a host loop with a stop
// read-back per launch (GDB_BARRIER_RELAUNCH) or a WHILE node
// (GDB_BARRIER_RELAUNCH_GRAPH).  `first` is the app state before the first
// step; `cap` bounds the launches.  Records the elapsed time and launch
// count in c->last; *steps_out (optional) = step launches run.
template <class... A>
inline int step_run(gdb_ctx* c, int kind, const void* init, const void* step, int grid, int block,
                    gdb::StepCtl* ctl, const gdb::StepCtl& first, unsigned long long cap,
                    bool run_steps, A... args) {
  gdb::StepCtl* h = (gdb::StepCtl*)pinned(c, sizeof(gdb::StepCtl));
  if (!h) return GDB_ERR_OOM;
  *h = first;
  h->done = 0;
  h->stop = run_steps ? 0 : 1;
  h->graph = kind == GDB_BARRIER_RELAUNCH_GRAPH ? 1 : 0;
  h->capped = 0;
  h->steps = 0;
  h->cap = cap;
  GDB_CUDA(c, cudaMemcpyAsync(ctl, h, sizeof(gdb::StepCtl), cudaMemcpyHostToDevice, c->stream));
  cudaGraphConditionalHandle cond = 0;
  gdb::StepCtl* ctl_arg = ctl;
  void* init_args[] = {(void*)&args..., nullptr};
  void* step_args[] = {(void*)&args..., (void*)&ctl_arg, (void*)&cond};
  unsigned long long launches = 1;
  if (kind == GDB_BARRIER_RELAUNCH || !run_steps) {
    GDB_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    GDB_CUDA(c, cudaLaunchKernel(init, grid, block, init_args, 0, c->stream));
    for (unsigned long long k = 0; run_steps && k < cap; ++k) {
      GDB_CUDA(c, cudaLaunchKernel(step, grid, block, step_args, 0, c->stream));
      ++launches;
      // the stop flag of the reference's relaunch loop
      GDB_CUDA(c, cudaMemcpyAsync(&h->stop, &ctl->stop, 4, cudaMemcpyDeviceToHost, c->stream));
      GDB_CUDA(c, cudaStreamSynchronize(c->stream));
      if (h->stop) break;
    }
    GDB_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  } else {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
    cudaGraphNode_t n_init = nullptr, n_cond = nullptr, n_step = nullptr;
    if (e == cudaSuccess) {
      cudaKernelNodeParams kp = {};
      kp.func = const_cast<void*>(init);
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
      kp.func = const_cast<void*>(step);
      kp.gridDim = dim3(grid);
      kp.blockDim = dim3(block);
      kp.kernelParams = step_args;
      e = cudaGraphAddKernelNode(&n_step, cp.conditional.phGraph_out[0], nullptr, 0, &kp);
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
  }
  GDB_CUDA(c, cudaMemcpyAsync(h, ctl, sizeof(gdb::StepCtl), cudaMemcpyDeviceToHost, c->stream));
  GDB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (h->capped || (run_steps && !h->stop))
    return set_error(c, GDB_ERR_TIMEOUT, "relaunch run exceeded its superstep bound");
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last.kernel_ms = ms;
  c->last.launches = (uint32_t)(kind == GDB_BARRIER_RELAUNCH_GRAPH ? 1 + h->steps : launches);
  c->last.participating = grid;
  c->last.launched = grid;
  return GDB_OK;
}

// CTAs of a step launch: every co-resident CTA of the step kernel (no
// discovery: a relaunched superstep never waits on another CTA).
inline int step_grid(gdb_ctx* c, const void* step, int block, int* grid) {
  int occ = 0;
  GDB_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, step, block, 0));
  *grid = std::max(1, occ) * c->sm_count;
  if (c->opt.max_ctas > 0) *grid = std::min(*grid, c->opt.max_ctas);
  return GDB_OK;
}

}  // namespace gdbi
