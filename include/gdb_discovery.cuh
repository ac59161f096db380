// gdb_discovery.cuh -- device API of the occupancy discovery protocol and
// the XF inter-CTA barrier for sm_103a.
//
// Replaces, for CUDA kernels, the reference's OpenCL device API
// (code/discovery_protocol/api/discovery.cl): DISCOVERY_PROTOCOL
// (:261-274) becomes `if (!gdb::discover(...)) return;`, discovery_barrier
// (:257, XF_barrier :177-238) becomes gdb::xf_barrier, p_get_* (:160-174)
// keep their names.  The shared state of discovery_kernel_ctx
// (code/discovery_protocol/api/common.h:33-48) is gdb::DeviceCtx, with every
// contended word and every barrier flag on its own 128-byte line.
//
// Every spin carries a %globaltimer deadline: on expiry the waiter records
// GDB_ERR_TIMEOUT in the context, raises the abort word, and all CTAs leave
// their waits -- a kernel using this header never hangs the GPU.  Memory
// ordering uses cuda::atomic_ref at device (gpu) scope: a slave's arrival is
// a release, the master's observation an acquire, and the master's release
// store publishes everything the whole grid wrote before the barrier.
#pragma once

#include <type_traits>

#include <cuda/atomic>
#include <stdint.h>

#include "gdb.h"

namespace gdb {

constexpr int kLineInts = 32;                 // one 128-byte line of ints
constexpr int kPollClosed = 0x40000000;       // lock-free poll: closed bit
constexpr int kPollCountMask = kPollClosed - 1;
constexpr unsigned kBarrierSpin = 4096;        // polls before a barrier wait backs off
constexpr int kArriveGroups = 16;              // combining XF: arrival counters
constexpr int kReleaseCopies = 4;              // combining XF: generation word copies

// discovery_kernel_ctx (common.h:33-48), one contended word per line.
struct __align__(128) DeviceCtx {
  int lock_counter;   int _p0[31];  // ticket dispenser / spin-lock word
  int lock_serving;   int _p1[31];  // now_serving
  int poll_word;      int _p2[31];  // lock-free poll: count | closed bit
  int kernel_counter; int _p3[31];  // CTAs through the closing phase
  int published;      int _p4[31];  // lock-free: participant count, 0 = not yet
  // protocol state touched under the lock (reference fields)
  int poll_open;      // prot_poll_open
  int prot_counter;   // prot_counter
  int num_participating;
  int skip;
  int _p5[28];
  // error reporting
  int status;         // first gdb_status recorded by the device (0 = OK)
  int abort;          // raised with any error: every spin gives up
  int err_where;      // code location of the first error
  int err_aux;
  int stall_after;    // test hook: master stops releasing after this many barriers (-1 off)
  int _p6[27];
  // broadcast release word of the epoch form of the XF barrier
  unsigned long long release;
  unsigned long long _p7[15];
  // combining form: slave s adds 1 to arrive[(s - 1) % kArriveGroups]; the
  // master zeroes them when its launch ends.  gen: release generation,
  // bumped once per barrier and never reset (waiters compare for change).
  struct {
    int v;
    int _p[31];
  } arrive[kArriveGroups];
  struct {
    unsigned v;
    int _p[31];
  } gen[kReleaseCopies];
  // flat form: every CTA adds 1 to one arrival counter and waits for the
  // barrier's count; the counter is never reset within a context, and the
  // master leaves its final value in flat_base for the next launch
  struct {
    unsigned v;
    int _p[31];
  } flat, flat_base;
};

// discovery_local_ctx (discovery.cl:19-23), in shared memory.
struct LocalCtx {
  int id;             // participating_group_id
  int P;              // participating_group_size
  int participating;  // is_participating
  int ok;             // 0 once this CTA saw an error / abort
  unsigned long long timeout_ns;  // limit of every single wait
  int barriers;       // barriers passed (master: for the stall test hook)
  unsigned gen;       // combining form: release generation last seen
  unsigned flat;      // flat form: the arrival count every CTA reached so far
  int stall_after;    // the context's stall test hook, read once per launch
};

// XF release forms.
enum XfRelease {
  kXfPerSlave = 0,   // the master stores 0 into every slave's flag (discovery.cl:155-161)
  kXfBroadcast = 1,  // slaves store a launch-unique epoch; one broadcast release word
  kXfCombined = 2,   // slaves add to 16 padded arrival counters; one generation word
  kXfFlat = 3,       // every CTA adds to one counter and waits for the barrier's count
  kXfAuto = 4        // flat up to kXfFlatMax participants, combining above
};

// Participants up to which the flat form is used.  In isolation (empty
// supersteps, every CTA arriving at once) it beats the combining form at
// every co-resident count of 512-thread CTAs (flat 1.21 / 1.26 / 1.39 /
// 1.53 us at 152 / 304 / 456 / 608, combining 2.02-2.05 us), and inside
// real kernels too (4096^2 grid BFS, 8,191 levels: 46.4 ms flat, 53.3 ms
// combining, with the earlier flat form); the one counter every CTA polls
// is its limit beyond a GPU's worth of CTAs.
constexpr int kXfFlatMax = 1024;

// The form a launch's barriers take (uniform: P is the same in every CTA).
__device__ __forceinline__ int xf_form(int release, int P) {
  return release == kXfAuto ? (P <= kXfFlatMax ? kXfFlat : kXfCombined) : release;
}

// Launch parameters every discovery kernel receives.
struct DiscoveryArgs {
  DeviceCtx* ctx;
  int* flags;              // flag_capacity lines of 32 ints
  int flag_capacity;
  int lock_kind;           // gdb_lock_kind
  int expected;            // CTAs the occupancy API says fit (0 = unknown)
  unsigned long long timeout_ns;
  unsigned long long close_wait_ns;  // lock-free: wait for `expected` pollers
  unsigned long long launch_id;      // > every earlier launch's: epochs never repeat
  int xf_release;                    // XfRelease
};

using aref = cuda::atomic_ref<int, cuda::thread_scope_device>;

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_acquire(int* p) {
  return aref(*p).load(cuda::memory_order_acquire);
}
__device__ __forceinline__ int ld_relaxed(int* p) {
  return aref(*p).load(cuda::memory_order_relaxed);
}
__device__ __forceinline__ void st_release(int* p, int v) {
  aref(*p).store(v, cuda::memory_order_release);
}
__device__ __forceinline__ void st_relaxed(int* p, int v) {
  aref(*p).store(v, cuda::memory_order_relaxed);
}
using aref64 = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>;
__device__ __forceinline__ unsigned long long ld_relaxed64(unsigned long long* p) {
  return aref64(*p).load(cuda::memory_order_relaxed);
}
__device__ __forceinline__ void fence_acq_rel_gpu() {
  cuda::atomic_thread_fence(cuda::memory_order_acq_rel, cuda::thread_scope_device);
}

// Record the first error and make every spinning CTA give up.
__device__ __forceinline__ void raise_error(DeviceCtx* c, int code, int where) {
  int expect = 0;
  if (aref(c->status).compare_exchange_strong(expect, code, cuda::memory_order_relaxed))
    st_relaxed(&c->err_where, where);
  aref(c->abort).store(1, cuda::memory_order_release);
}

// Bounded spin: returns false on abort, or when this wait has lasted
// longer than timeout_ns (then GDB_ERR_TIMEOUT is recorded with `where`).
// The clock is read only once a wait is not over after a few polls.
// `pure` polls spin without sleeping (barrier waits are short when every
// CTA is resident), after which __nanosleep backs the poller off.
template <class Done>
__device__ __forceinline__ bool spin_until(DeviceCtx* c, unsigned long long timeout_ns,
                                           int where, Done done, unsigned pure = 32) {
  unsigned ns = 0;
  unsigned long long deadline = 0;
  for (unsigned k = 1;; ++k) {
    if (done()) return true;
    if ((k & 15) == 0) {
      if (ld_relaxed(&c->abort)) return false;
      const unsigned long long now = globaltimer();
      if (deadline == 0) {
        deadline = now + timeout_ns;
      } else if (now > deadline) {
        raise_error(c, GDB_ERR_TIMEOUT, where);
        return false;
      }
    }
    if (k > pure) {
      __nanosleep(ns);
      ns = ns < 128 ? ns + 16 : 128;
    }
  }
}

// ------------------------------------------------------------------ locks
// Ticket lock (locks.cl:25-34) and exchange spin lock (locks.cl:11-20).
__device__ __forceinline__ bool lock_acquire(DeviceCtx* c, int kind,
                                             unsigned long long timeout_ns) {
  if (kind == GDB_LOCK_SPIN) {
    return spin_until(c, timeout_ns, 1, [&] {
      return aref(c->lock_counter).exchange(1, cuda::memory_order_acq_rel) == 0;
    });
  }
  const int ticket = aref(c->lock_counter).fetch_add(1, cuda::memory_order_acq_rel);
  return spin_until(c, timeout_ns, 2, [&] { return ld_acquire(&c->lock_serving) == ticket; });
}
__device__ __forceinline__ void lock_release(DeviceCtx* c, int kind) {
  if (kind == GDB_LOCK_SPIN) {
    st_release(&c->lock_counter, 0);
  } else {
    const int s = ld_relaxed(&c->lock_serving);
    st_release(&c->lock_serving, s + 1);
  }
}

// reset_kernel_context (discovery.cl:31-37): re-arm for the next launch.
// Called by the last CTA through while it holds the lock; the final release
// of the lock words is the implicit unlock.
__device__ __forceinline__ void reset_kernel_context(DeviceCtx* c) {
  st_relaxed(&c->poll_open, 1);
  st_relaxed(&c->prot_counter, 0);
  st_relaxed(&c->kernel_counter, 0);
  st_release(&c->lock_counter, 0);
  st_release(&c->lock_serving, 0);
}

// discovery_protocol_master (discovery.cl:42-88) with a mutex, executed by
// one thread per CTA.
__device__ inline void protocol_master_locked(const DiscoveryArgs& a, LocalCtx* l) {
  DeviceCtx* c = a.ctx;
  const int kind = a.lock_kind;
  // polling phase
  if (!lock_acquire(c, kind, l->timeout_ns)) { l->ok = 0; l->participating = 0; return; }
  if (ld_relaxed(&c->poll_open)) {
    const int id = ld_relaxed(&c->prot_counter);
    l->participating = 1;
    l->id = id;
    st_relaxed(&c->prot_counter, id + 1);
  } else {
    l->participating = 0;
  }
  lock_release(c, kind);
  // closing phase
  if (!lock_acquire(c, kind, l->timeout_ns)) { l->ok = 0; l->participating = 0; return; }
  const int kc = ld_relaxed(&c->kernel_counter) + 1;
  st_relaxed(&c->kernel_counter, kc);
  const bool reset = kc == (int)gridDim.x;
  if (ld_relaxed(&c->poll_open)) {
    st_relaxed(&c->poll_open, 0);
    st_relaxed(&c->num_participating, ld_relaxed(&c->prot_counter));
  }
  l->P = ld_relaxed(&c->prot_counter);
  if (reset) reset_kernel_context(c);
  else lock_release(c, kind);
}

// Lock-free protocol: one fetch_add polls (the returned count is the id
// unless the closed bit is set), the first participant through the closing
// step sets the closed bit with fetch_or and publishes the count it saw.
// When the occupancy API's figure `expected` is known, participants keep
// the poll open until that many CTAs have polled or close_wait_ns passed,
// so CTAs that start a little later are still discovered.
__device__ inline void protocol_master_lockfree(const DiscoveryArgs& a, LocalCtx* l) {
  DeviceCtx* c = a.ctx;
  const int old = aref(c->poll_word).fetch_add(1, cuda::memory_order_acq_rel);
  if (old & kPollClosed) {
    l->participating = 0;
  } else {
    l->participating = 1;
    l->id = old & kPollCountMask;
    if (a.expected > 0) {
      const unsigned long long until = globaltimer() + a.close_wait_ns;
      unsigned ns = 0;
      for (;;) {
        const int w = ld_relaxed(&c->poll_word);
        if ((w & kPollClosed) || (w & kPollCountMask) >= a.expected) break;
        if (globaltimer() > until || ld_relaxed(&c->abort)) break;
        __nanosleep(ns);
        ns = ns < 256 ? ns + 32 : 256;
      }
    }
    const int prev = aref(c->poll_word).fetch_or(kPollClosed, cuda::memory_order_acq_rel);
    if (!(prev & kPollClosed)) {
      const int P = prev & kPollCountMask;
      st_relaxed(&c->num_participating, P);
      st_release(&c->published, P);
      l->P = P;
    } else {
      int P = 0;
      if (!spin_until(c, l->timeout_ns, 3, [&] { return (P = ld_acquire(&c->published)) != 0; })) {
        l->ok = 0;
        l->participating = 0;
      }
      l->P = P;
    }
  }
  // the last CTA through re-arms the context for the next launch
  const int k = aref(c->kernel_counter).fetch_add(1, cuda::memory_order_acq_rel);
  if (k == (int)gridDim.x - 1) {
    st_relaxed(&c->published, 0);
    st_relaxed(&c->poll_word, 0);
    st_release(&c->kernel_counter, 0);
  }
}

// DISCOVERY_PROTOCOL (discovery.cl:213-226).  All threads of the CTA call
// it; returns true for participating CTAs (the others must return).
__device__ inline bool discover(const DiscoveryArgs& a, LocalCtx* l) {
  if (threadIdx.x == 0) {
    l->ok = 1;
    l->barriers = 0;
    l->timeout_ns = a.timeout_ns;
    DeviceCtx* c = a.ctx;
    if (ld_relaxed(&c->skip)) {
      l->P = gridDim.x;
      l->participating = 1;
      l->id = blockIdx.x;
      if (blockIdx.x == 0) st_relaxed(&c->num_participating, gridDim.x);
    } else if (a.lock_kind == GDB_LOCK_FREE) {
      protocol_master_lockfree(a, l);
    } else {
      protocol_master_locked(a, l);
    }
    if (l->participating &&
        (l->P > a.flag_capacity || l->P - 1 > 32 * (int)blockDim.x)) {
      raise_error(c, GDB_ERR_CAPACITY, 4);
      l->ok = 0;
    }
    if (!l->ok) l->participating = 0;
    // combining XF: no release can happen before this CTA's first arrival
    l->gen = (unsigned)ld_relaxed((int*)&c->gen[0].v);
    // flat XF: the count the previous launch ended at
    l->flat = (unsigned)ld_relaxed((int*)&c->flat_base.v);
    // set by the host between launches: read once, not at every barrier
    l->stall_after = ld_relaxed(&c->stall_after);
  }
  __syncthreads();
  return l->participating != 0;
}

// p_get_* (discovery.cl:112-126)
__device__ __forceinline__ int p_get_group_id(const LocalCtx* l) { return l->id; }
__device__ __forceinline__ int p_get_num_groups(const LocalCtx* l) { return l->P; }
__device__ __forceinline__ int p_get_global_id(const LocalCtx* l) {
  return threadIdx.x + blockDim.x * l->id;
}
__device__ __forceinline__ int p_get_global_size(const LocalCtx* l) {
  return l->P * blockDim.x;
}

// A barrier hook that does nothing (see xf_barrier).
struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

// Warp-uniform bounded spin: done() must return the same value in every
// lane; lane 0 watches the abort word and the deadline for the warp.
template <class Done>
__device__ __forceinline__ bool spin_until_warp(DeviceCtx* c, unsigned long long timeout_ns,
                                                int where, Done done, unsigned pure) {
  unsigned ns = 0;
  unsigned long long deadline = 0;
  for (unsigned k = 1;; ++k) {
    if (done()) return true;
    if ((k & 15) == 0) {
      int stop = 0;
      if ((threadIdx.x & 31) == 0) {
        if (ld_relaxed(&c->abort)) {
          stop = 1;
        } else {
          const unsigned long long now = globaltimer();
          if (deadline == 0) {
            deadline = now + timeout_ns;
          } else if (now > deadline) {
            raise_error(c, GDB_ERR_TIMEOUT, where);
            stop = 1;
          }
        }
      }
      if (__shfl_sync(0xffffffffu, stop, 0)) return false;
    }
    if (k > pure) {
      __nanosleep(ns);
      ns = ns < 128 ? ns + 16 : 128;
    }
  }
}

// Combining form of the XF barrier.  The master/slave roles stay, but the
// master no longer polls one padded flag per slave: slave s adds 1 to the
// padded counter arrive[(s - 1) % 16] (fence + relaxed add: a release),
// and the master's first warp watches the 16 counters (acquire loads)
// until each holds (barrier + 1) x its group size.  The release is a
// generation word bumped by the master (fence + relaxed store), written
// to four padded copies so that each copy is polled (acquire loads) by a
// quarter of the slaves.  Nothing has to be reset between
// barriers: counts grow within a launch (the master zeroes them when it
// leaves the launch, see xf_finish) and the generation only ever changes,
// so captured launches can be replayed.
template <class Hook>
__device__ inline bool xf_barrier_combined(const DiscoveryArgs& a, LocalCtx* l, Hook&& hook) {
  DeviceCtx* c = a.ctx;
  int ok = 1;
  if (l->id == 0) {
    // no CTA barrier first: warp 0 starts watching at once, and the
    // __syncthreads_and below holds the release until the whole master
    // CTA has arrived
    const int slaves = l->P - 1;
    if (threadIdx.x < 32 && slaves > 0) {
      const int lane = threadIdx.x;
      const int n_g = lane < kArriveGroups
                          ? slaves / kArriveGroups + (lane < slaves % kArriveGroups ? 1 : 0)
                          : 0;
      const int target = (l->barriers + 1) * n_g;
      bool mine = n_g == 0;
      ok = spin_until_warp(c, l->timeout_ns, 5, [&] {
        if (!mine) mine = (int)((unsigned)ld_acquire(&c->arrive[lane].v) - (unsigned)target) >= 0;
        return __all_sync(0xffffffffu, mine);
      }, kBarrierSpin);
    }
    ok = __syncthreads_and(ok);
    if (ok && l->stall_after >= 0 && l->barriers >= l->stall_after) {
      if (threadIdx.x == 0) spin_until(c, l->timeout_ns, 6, [&] { return false; });
      ok = 0;
    }
    if (ok) {
      if constexpr (!std::is_same<typename std::decay<Hook>::type, NoHook>::value) {
        hook();
        __syncthreads();
      }
      if (threadIdx.x < kReleaseCopies) {
        fence_acq_rel_gpu();  // release: the grid's writes before the generation
        aref(*(int*)&c->gen[threadIdx.x].v).store((int)(l->gen + 1), cuda::memory_order_relaxed);
      }
      __syncwarp();
      if (threadIdx.x == 0) l->gen += 1;
    }
  } else {
    __syncthreads();
    if (threadIdx.x == 0) {
      const int g0 = (int)l->gen;
      fence_acq_rel_gpu();  // release: this CTA's writes before its arrival
      aref(c->arrive[(l->id - 1) % kArriveGroups].v).fetch_add(1, cuda::memory_order_relaxed);
      int* word = (int*)&c->gen[l->id % kReleaseCopies].v;
      ok = spin_until(c, l->timeout_ns, 7, [&] { return ld_acquire(word) != g0; }, kBarrierSpin);
      if (ok) l->gen = (unsigned)(g0 + 1);  // one bump per barrier
      else l->ok = 0;
      l->barriers++;
    }
    // one CTA barrier between the release and the slave's next superstep
    __syncthreads();
    return l->ok != 0;
  }
  if (threadIdx.x == 0) {
    if (!ok) l->ok = 0;
    l->barriers++;
  }
  __syncthreads();
  return l->ok != 0;
}

// End of a launch.  Combining form: the master zeroes the arrival counts
// (every arrival of its last barrier has been counted, and no CTA arrives
// again).  Flat form: the master records the count reached, which the next
// launch's CTAs start from (CTAs still polling this launch's last barrier
// read the counter, not this word).  After an error the host re-arms the
// context.
__device__ inline void xf_finish(const DiscoveryArgs& a, const LocalCtx* l) {
  if (!l->participating || l->id != 0 || !l->ok) return;
  const int form = xf_form(a.xf_release, l->P);
  if (form == kXfCombined && threadIdx.x < kArriveGroups)
    st_relaxed(&a.ctx->arrive[threadIdx.x].v, 0);
  if (form == kXfFlat && threadIdx.x == 0) st_relaxed((int*)&a.ctx->flat_base.v, (int)l->flat);
}

// Flat form: thread 0 of every CTA adds 1 to the arrival counter with one
// acquire-release atomic that returns the count before it, and polls the
// counter (acquire) until it holds this barrier's count -- one round trip
// after the last arrival, as a grid-wide counter barrier.  The returned
// count matters twice:
// - the last arrival sees that it is last and does not poll (its atomic
//   acquires every earlier arrival's release);
// - a CTA starts polling only once its add has come back, so the polls do
//   not crowd the counter's line while the adds are still landing.
// Per barrier, this form against the fence + relaxed add + immediate
// polls it replaces, and against cooperative_groups grid.sync
// (gdb_barrier_bench, empty supersteps, 512-thread CTAs, the same box):
// | CTAs | this form | fence + relaxed add | grid.sync |
// |---|---|---|---|
// | 152 | 1.21 us | 1.23 | 1.15 |
// | 304 | 1.26 | 1.40 | 1.18 |
// | 456 | 1.39 | 1.72 | 1.18 |
// | 608 | 1.53 | 2.29 | 1.56 |
// A hook (or the stall test hook) makes the master arrive last: it waits
// for the other P - 1, runs the hook, then arrives.
template <class Hook>
__device__ inline bool xf_barrier_flat(const DiscoveryArgs& a, LocalCtx* l, Hook&& hook) {
  DeviceCtx* c = a.ctx;
  constexpr bool hooked = !std::is_same<typename std::decay<Hook>::type, NoHook>::value;
  int* counter = (int*)&c->flat.v;
  const unsigned target = l->flat + (unsigned)l->P;
  int ok = 1;
  __syncthreads();
  if (l->id == 0 && (hooked || l->stall_after >= 0)) {
    if (threadIdx.x == 0)
      ok = spin_until(c, l->timeout_ns, 5, [&] {
        return (int)((unsigned)ld_acquire(counter) - (target - 1u)) >= 0;
      }, kBarrierSpin);
    ok = __syncthreads_and(ok);
    if (ok && l->stall_after >= 0 && l->barriers >= l->stall_after) {
      // test hook: never arrive; every other CTA's wait must end with
      // GDB_ERR_TIMEOUT at its deadline
      if (threadIdx.x == 0) spin_until(c, l->timeout_ns, 6, [&] { return false; });
      ok = 0;
    }
    if (ok) {
      if constexpr (hooked) {
        hook();
        __syncthreads();
      }
      // release: the grid's writes (acquired above) before the last arrival
      if (threadIdx.x == 0) aref(*counter).fetch_add(1, cuda::memory_order_release);
    }
  } else if (threadIdx.x == 0) {
    // release: this CTA's writes before its arrival; acquire: when it is
    // the last, every other CTA's writes before the superstep goes on
    const unsigned before = (unsigned)aref(*counter).fetch_add(1, cuda::memory_order_acq_rel);
    if ((int)(before + 1u - target) < 0)
      ok = spin_until(c, l->timeout_ns, 7, [&] {
        return (int)((unsigned)ld_acquire(counter) - target) >= 0;
      }, kBarrierSpin);
  }
  if (threadIdx.x == 0) {
    if (!ok) l->ok = 0;
    l->barriers++;
    l->flat = target;
  }
  __syncthreads();
  return l->ok != 0;
}

// XF barrier (discovery.cl:129-190) over the participating CTAs.  Slave: one
// elected thread publishes its arrival in its own padded flag and spins
// until released.  Master: each thread issues loads for all of its peers'
// flags at once and retires the ones that arrived, so the wait costs one
// L2 round trip after the last arrival; then a CTA barrier and the
// release.  Two release forms (DiscoveryArgs::xf_release):
//  * per-slave: arrival stores 1, the master stores 0 into every flag
//    (the reference's form);
//  * broadcast: arrival stores the barrier's epoch (launch id << 32 |
//    barrier count, never repeated), the master stores the epoch once into
//    a broadcast word every slave polls -- no per-slave stores, no resets.
// Ordering: fence.acq_rel.gpu + relaxed store on the releasing side,
// relaxed polls + fence.acq_rel.gpu on the acquiring side, CTA barriers
// in between.  Returns false (uniformly across the CTA) after an error or
// a timeout anywhere in the grid.
//
// `hook` runs in the master CTA (every thread calls it) after every
// participant has arrived and before the release: it sees all the grid's
// writes of the superstep, and its own writes are published by the release
// (a superstep-boundary decision taken once, e.g. the schedule selector).
template <class Hook>
__device__ inline bool xf_barrier(const DiscoveryArgs& a, LocalCtx* l, Hook&& hook) {
  const int form = xf_form(a.xf_release, l->P);
  if (form == kXfCombined) return xf_barrier_combined(a, l, hook);
  if (form == kXfFlat) return xf_barrier_flat(a, l, hook);
  DeviceCtx* c = a.ctx;
  const int P = l->P;
  const bool bcast = a.xf_release == kXfBroadcast;
  const unsigned long long tag = (a.launch_id << 32) | (unsigned)(l->barriers + 1);
  int ok = 1;
  if (l->id == 0) {
    __syncthreads();
    // up to 32 peers per thread (P <= 32 * blockDim.x + 1 is checked by the host)
    unsigned pending = 0;
    int k = 0;
    for (int peer = threadIdx.x + 1; peer < P; peer += blockDim.x, ++k) pending |= 1u << k;
    if (pending) {
      ok = spin_until(c, l->timeout_ns, 5, [&] {
        int kk = 0;
        for (int peer = threadIdx.x + 1; peer < P; peer += blockDim.x, ++kk) {
          if ((pending >> kk) & 1u) {
            int* f = &a.flags[(size_t)peer * kLineInts];
            const bool arrived = bcast ? ld_relaxed64((unsigned long long*)f) >= tag
                                       : ld_relaxed(f) != 0;
            if (arrived) pending &= ~(1u << kk);
          }
        }
        return pending == 0;
      }, kBarrierSpin);
      fence_acq_rel_gpu();  // acquire: the slaves' writes before ours
    }
    ok = __syncthreads_and(ok);
    if (ok && l->stall_after >= 0 && l->barriers >= l->stall_after) {
      // test hook: never release; wait on a word nobody sets until the
      // deadline, which must end every CTA's wait with GDB_ERR_TIMEOUT
      if (threadIdx.x == 0) {
        spin_until(c, l->timeout_ns, 6, [&] { return false; });
      }
      ok = 0;
    }
    if (ok) {
      if constexpr (!std::is_same<typename std::decay<Hook>::type, NoHook>::value) {
        hook();
        __syncthreads();
      }
      if (bcast) {
        if (threadIdx.x == 0) {
          fence_acq_rel_gpu();  // release: the grid's writes before the word
          aref64(c->release).store(tag, cuda::memory_order_relaxed);
        }
      } else {
        fence_acq_rel_gpu();  // release: publish the grid's writes with the flags
        for (int peer = threadIdx.x + 1; peer < P; peer += blockDim.x)
          st_relaxed(&a.flags[(size_t)peer * kLineInts], 0);
      }
    }
  } else {
    __syncthreads();
    if (threadIdx.x == 0) {
      int* f = &a.flags[(size_t)l->id * kLineInts];
      fence_acq_rel_gpu();
      if (bcast) {
        aref64(*(unsigned long long*)f).store(tag, cuda::memory_order_relaxed);
        ok = spin_until(c, l->timeout_ns, 7, [&] { return ld_relaxed64(&c->release) >= tag; },
                        kBarrierSpin);
      } else {
        st_relaxed(f, 1);
        ok = spin_until(c, l->timeout_ns, 7, [&] { return ld_relaxed(f) == 0; }, kBarrierSpin);
      }
      fence_acq_rel_gpu();
      l->ok = ok;
    }
    __syncthreads();
    ok = l->ok;
  }
  // every CTA leaves together on error
  if (threadIdx.x == 0) {
    if (!ok) l->ok = 0;
    l->barriers++;
  }
  __syncthreads();
  return l->ok != 0;
}

__device__ inline bool xf_barrier(const DiscoveryArgs& a, LocalCtx* l) {
  return xf_barrier(a, l, NoHook{});
}

}  // namespace gdb
