// Opaque handle definitions shared by the C ABI translation units (internal to libgbpt).
#pragma once

#include <mutex>
#include <string>

#include "../../include/gbpt.h"
#include "trace_kernels.h"

// Device staging of the host-buffer trace entry points, kept with the BVH and reused by every
// call (grown when a larger batch arrives): rays, last_prim and results of the whole batch, one
// side stream and the events that order the chunk pipeline against the caller's stream.
struct HostTraceStaging
{
    std::mutex mu;            // one host-buffer call at a time per BVH
    char* buf = nullptr;
    size_t cap = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t start = nullptr, side_done = nullptr;
};

struct gbpt_bvh
{
    gbpt::DeviceBVH dev;
    gbpt_bvh_stats stats;
    int device = 0;
    gbpt::TraceConfig cfg[2] = {gbpt::default_trace_config(false), gbpt::default_trace_config(true)};
    mutable HostTraceStaging staging;
};

namespace gbpt {
// Records the message for gbpt_last_error() on this thread and returns s.
gbpt_status set_error(gbpt_status s, const std::string& msg);
gbpt_status cuda_error(cudaError_t e, const char* what);
}  // namespace gbpt
