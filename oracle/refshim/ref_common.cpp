// Work-item state for the OpenCL C shim (test infrastructure).
#include "opencl_shim.h"
thread_local shim_workitem shim_wi = {0, 0, 0, 1, 1, 1};
