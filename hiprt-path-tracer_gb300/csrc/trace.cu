// Closest-hit and any-hit traversal kernels of the 8-wide compressed BVH (sm_103a).
// The per-ray traversal lives in trace_core.h; this file holds the launches: one thread per ray,
// 16-byte ray/hit records loaded and stored as single 128-bit accesses.
#include <cuda_runtime.h>
#include <stdint.h>

#include "trace_core.h"
#include "trace_kernels.h"

namespace gbpt {
namespace {

template <bool ANY_HIT, bool COUNT>
__global__ void __launch_bounds__(128) trace_kernel(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                                    const float4* __restrict__ origin_tmin,
                                                    const float4* __restrict__ dir_tmax,
                                                    const int32_t* __restrict__ last_prim, int64_t n_rays,
                                                    float4* __restrict__ hits, uint8_t* __restrict__ occluded,
                                                    unsigned long long* __restrict__ counters)
{
    const int64_t ray = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ray >= n_rays) return;
    const float4 ot = origin_tmin[ray];
    const float4 dt = dir_tmax[ray];
    const int32_t skip_prim = last_prim ? last_prim[ray] : -1;
    uint32_t n_nodes = 0, n_tris = 0;
    const float4 h = core::trace_ray<ANY_HIT, COUNT>(nodes, tris, ot, dt, skip_prim, n_nodes, n_tris);
    if (ANY_HIT)
    {
        if (occluded) occluded[ray] = __float_as_int(h.w) >= 0 ? 1 : 0;
    }
    else if (hits)
        hits[ray] = h;

    if (COUNT)
    {
        const unsigned m = __activemask();
        const unsigned sn = __reduce_add_sync(m, n_nodes);
        const unsigned st = __reduce_add_sync(m, n_tris);
        if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1))
        {
            atomicAdd(counters + 0, (unsigned long long)sn);
            atomicAdd(counters + 1, (unsigned long long)st);
        }
    }
}

}  // namespace

cudaError_t launch_trace(const DeviceBVH& bvh, const float* origin_tmin, const float* dir_tmax,
                         const int32_t* last_prim, int64_t n_rays, float* hits, uint8_t* occluded, bool any_hit,
                         unsigned long long* counters, cudaStream_t stream)
{
    if (n_rays <= 0) return cudaSuccess;
    const int threads = 128;
    const int64_t blocks = (n_rays + threads - 1) / threads;
    const uint4* nodes = reinterpret_cast<const uint4*>(bvh.nodes);
    const float4* tris = reinterpret_cast<const float4*>(bvh.tris);
    const float4* o = reinterpret_cast<const float4*>(origin_tmin);
    const float4* d = reinterpret_cast<const float4*>(dir_tmax);
    float4* h = reinterpret_cast<float4*>(hits);
    if (counters)
    {
        if (any_hit)
            trace_kernel<true, true><<<(unsigned)blocks, threads, 0, stream>>>(nodes, tris, o, d, last_prim, n_rays, h,
                                                                               occluded, counters);
        else
            trace_kernel<false, true><<<(unsigned)blocks, threads, 0, stream>>>(nodes, tris, o, d, last_prim, n_rays, h,
                                                                                occluded, counters);
    }
    else if (any_hit)
        trace_kernel<true, false><<<(unsigned)blocks, threads, 0, stream>>>(nodes, tris, o, d, last_prim, n_rays, h,
                                                                            occluded, nullptr);
    else
        trace_kernel<false, false><<<(unsigned)blocks, threads, 0, stream>>>(nodes, tris, o, d, last_prim, n_rays, h,
                                                                             occluded, nullptr);
    return cudaGetLastError();
}

}  // namespace gbpt
