// Launch interface of the traversal kernels (internal to libgbpt).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbpt {

struct DeviceBVH
{
    const void* nodes = nullptr;  // WideNode[n_nodes]
    const void* tris = nullptr;   // float4[3 * n_tris]
    int64_t n_nodes = 0;
    int64_t n_tris = 0;
    int32_t depth = 0;  // wide depth (bounds the traversal stack's node groups)
};

// Launch configuration of a traversal (the fields of gbpt_trace_config)
constexpr int kTraceKernelPerRay = 1;      // one thread per ray
constexpr int kTraceKernelPersistent = 2;  // persistent warps with lane refill and triangle postponing
constexpr int kTraceKernelFetch = 3;       // persistent warps, each lane fetching its next ray when done
struct TraceConfig
{
    int32_t kernel;
    int32_t block;           // threads per block
    int32_t refill_below;    // persistent: refill when fewer lanes than this trace
    int32_t postpone_below;  // persistent: triangle steps need at least this many lanes
    int32_t blocks_per_sm;   // persistent grid
    int32_t shared_stack;    // traversal-stack entries per thread in shared memory (0, 8 or 16)
    int32_t triangle_test;   // core::kTriMollerTrumbore (parity) or core::kTriWatertight
    int32_t top_levels;      // 1: the 73 nodes nearest the root staged in shared memory per block
};

TraceConfig default_trace_config(bool any_hit);
bool valid_trace_config(const TraceConfig& c);

// cfg == nullptr: default_trace_config(any_hit). counters != nullptr: the counting per-ray kernel.
cudaError_t launch_trace(const DeviceBVH& bvh, const float* origin_tmin, const float* dir_tmax,
                         const int32_t* last_prim, int64_t n_rays, float* hits, uint8_t* occluded, bool any_hit,
                         unsigned long long* counters, cudaStream_t stream, const TraceConfig* cfg = nullptr);

}  // namespace gbpt
