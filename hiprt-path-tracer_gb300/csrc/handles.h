// Opaque handle definitions shared by the C ABI translation units (internal to libgbpt).
#pragma once

#include <string>

#include "../../include/gbpt.h"
#include "trace_kernels.h"

struct gbpt_bvh
{
    gbpt::DeviceBVH dev;
    gbpt_bvh_stats stats;
    int device = 0;
    gbpt::TraceConfig cfg[2] = {gbpt::default_trace_config(false), gbpt::default_trace_config(true)};
};

namespace gbpt {
// Records the message for gbpt_last_error() on this thread and returns s.
gbpt_status set_error(gbpt_status s, const std::string& msg);
gbpt_status cuda_error(cudaError_t e, const char* what);
}  // namespace gbpt
