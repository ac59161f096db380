// Driver: the reference's discovery protocol and XF barrier
// (code/discovery_protocol/api/discovery.cl, included by path) executed by
// `groups` host threads, one work-group of one work-item each.  Records the
// participating id each group obtained (-1 for groups that left), the
// number of participating groups, and whether the context was left reset
// for the next launch.  Test infrastructure.
#include <thread>
#include <vector>
#include "opencl_shim.h"

namespace disc {
#include "discovery.cl"

// The reference's occupancy kernel run_test (occupancy_test.cl:8-17) plus a
// record of the id each group was given and `rounds` XF barriers during
// which every participant increments a shared counter.
void recorded_test(__global discovery_kernel_ctx* gl_ctx, int* ids,
                   int rounds, int* counter, int* errors) {
  DISCOVERY_PROTOCOL(gl_ctx);
  ids[get_group_id(0)] = p_get_group_id(gl_ctx, &local_ctx);
  int n = p_get_num_groups(gl_ctx, &local_ctx);
  for (int r = 0; r < rounds; ++r) {
    atomic_add(counter, 1);
    discovery_barrier(gl_ctx, &local_ctx);
    // after the r-th barrier every participant has added r+1 times
    if (atomic_load_explicit(counter, memory_order_relaxed,
                             memory_scope_device) < (r + 1) * n)
      atomic_add(errors, 1);
    discovery_barrier(gl_ctx, &local_ctx);
  }
}
}  // namespace disc

extern "C" int ref_discovery_threads(int groups, int rounds, int* ids_out,
                                     int* num_participating_out,
                                     int* reset_ok_out, int* errors_out) {
  disc::discovery_kernel_ctx ctx;
  shim_single([&] { disc::init_discovery_kernel_ctx(&ctx, 0); });
  std::vector<int> ids(groups, -1);
  int counter = 0, errors = 0;
  std::vector<std::thread> th;
  for (int g = 0; g < groups; ++g) {
    th.emplace_back([&, g] {
      shim_wi = shim_workitem{(size_t)g, 0, (size_t)g, (size_t)groups, 1,
                              (size_t)groups};
      disc::recorded_test(&ctx, ids.data(), rounds, &counter, &errors);
    });
  }
  for (auto& t : th) t.join();
  for (int g = 0; g < groups; ++g) ids_out[g] = ids[g];
  *num_participating_out = ctx.num_participating;
  *reset_ok_out = ctx.prot_poll_open == 1 && ctx.prot_counter == 0 &&
                  ctx.kernel_counter == 0 && ctx.m.counter == 0 &&
                  ctx.m.now_serving == 0;
  *errors_out = errors;
  return 0;
}
