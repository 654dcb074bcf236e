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
};

cudaError_t launch_trace(const DeviceBVH& bvh, const float* origin_tmin, const float* dir_tmax,
                         const int32_t* last_prim, int64_t n_rays, float* hits, uint8_t* occluded, bool any_hit,
                         unsigned long long* counters, cudaStream_t stream);

}  // namespace gbpt
