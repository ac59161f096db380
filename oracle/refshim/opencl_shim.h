// OpenCL C -> C++ shim: lets the reference's own .cl kernel sources be
// compiled with g++ and executed on host threads, so the CPU oracle can be
// pinned against the reference's code itself.
//
// TEST INFRASTRUCTURE ONLY (force-included by oracle/refshim/Makefile; the
// reference sources are included by path from the reference checkout and
// never copied).
//
// Execution model: a "work-item" is a host thread; its NDRange coordinates
// live in a thread_local record that the drivers set before calling a
// kernel function.  Work-groups have one work-item each, so barrier() is a
// no-op and local memory is ordinary stack memory.  Atomics are real
// (__atomic builtins, sequentially consistent), so several host threads
// can run the discovery protocol and XF barrier as separate work-groups.
#pragma once

#include <stddef.h>
#include <stdint.h>

// address-space and function qualifiers
#define __kernel
#define kernel
#define __global
#define __local
#define __constant const

typedef unsigned int uint;
typedef int atomic_int;
typedef unsigned int cl_mem_fence_flags;

#define CLK_LOCAL_MEM_FENCE 1u
#define CLK_GLOBAL_MEM_FENCE 2u

typedef enum {
  memory_order_relaxed,
  memory_order_acquire,
  memory_order_release,
  memory_order_acq_rel,
  memory_order_seq_cst
} memory_order;
typedef enum { memory_scope_work_group, memory_scope_device } memory_scope;

struct shim_workitem {
  size_t gid, lid, grp, ngroups, lsize, gsize;
};
extern thread_local shim_workitem shim_wi;

static inline size_t get_global_id(uint) { return shim_wi.gid; }
static inline size_t get_local_id(uint) { return shim_wi.lid; }
static inline size_t get_group_id(uint) { return shim_wi.grp; }
static inline size_t get_num_groups(uint) { return shim_wi.ngroups; }
static inline size_t get_local_size(uint) { return shim_wi.lsize; }
static inline size_t get_global_size(uint) { return shim_wi.gsize; }

static inline void barrier(cl_mem_fence_flags) {}
static inline void mem_fence(cl_mem_fence_flags) {
  __atomic_thread_fence(__ATOMIC_SEQ_CST);
}

// OpenCL 2.0 atomics used by the discovery protocol and XF barrier.
static inline void atomic_store_explicit(volatile int* p, int v, memory_order,
                                         memory_scope) {
  __atomic_store_n(p, v, __ATOMIC_SEQ_CST);
}
static inline int atomic_load_explicit(volatile int* p, memory_order,
                                       memory_scope) {
  return __atomic_load_n(p, __ATOMIC_SEQ_CST);
}
static inline int atomic_fetch_add_explicit(volatile int* p, int v,
                                            memory_order, memory_scope) {
  return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}
static inline int atomic_exchange_explicit(volatile int* p, int v,
                                           memory_order, memory_scope) {
  return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST);
}
static inline void atomic_work_item_fence(cl_mem_fence_flags, memory_order,
                                          memory_scope) {
  __atomic_thread_fence(__ATOMIC_SEQ_CST);
}

// OpenCL 1.x atomics (int and uint overloads).
#define SHIM_ATOMICS(T)                                                     \
  static inline T atomic_add(volatile T* p, T v) {                           \
    return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);                       \
  }                                                                          \
  static inline T atomic_sub(volatile T* p, T v) {                           \
    return __atomic_fetch_sub(p, v, __ATOMIC_SEQ_CST);                       \
  }                                                                          \
  static inline T atomic_xchg(volatile T* p, T v) {                          \
    return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST);                      \
  }                                                                          \
  static inline T atomic_min(volatile T* p, T v) {                           \
    T old = __atomic_load_n(p, __ATOMIC_SEQ_CST);                            \
    while (v < old &&                                                        \
           !__atomic_compare_exchange_n(p, &old, v, false, __ATOMIC_SEQ_CST, \
                                        __ATOMIC_SEQ_CST)) {                 \
    }                                                                        \
    return old;                                                              \
  }                                                                          \
  static inline T atomic_cmpxchg(volatile T* p, T cmp, T v) {                \
    __atomic_compare_exchange_n(p, &cmp, v, false, __ATOMIC_SEQ_CST,         \
                                __ATOMIC_SEQ_CST);                           \
    return cmp;                                                              \
  }
SHIM_ATOMICS(int)
SHIM_ATOMICS(unsigned int)
#undef SHIM_ATOMICS

// Run a barrier-free NDRange kernel as a sequential loop over global ids.
template <typename F>
static inline void shim_ndrange(size_t global, size_t local, F&& body) {
  shim_workitem saved = shim_wi;
  for (size_t g = 0; g < global; ++g) {
    shim_wi.gid = g;
    shim_wi.lid = g % local;
    shim_wi.grp = g / local;
    shim_wi.ngroups = (global + local - 1) / local;
    shim_wi.lsize = local;
    shim_wi.gsize = global;
    body();
  }
  shim_wi = saved;
}

// Run a kernel as one work-group of one work-item (persistent kernels).
template <typename F>
static inline void shim_single(F&& body) {
  shim_workitem saved = shim_wi;
  shim_wi = shim_workitem{0, 0, 0, 1, 1, 1};
  body();
  shim_wi = saved;
}
