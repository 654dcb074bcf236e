// Closest-hit and any-hit traversal kernels of the 8-wide compressed BVH (sm_103a).
//
// The production kernels are persistent warps: each warp owns the groups of 32 consecutive rays
// g = warp, warp + n_warps, ... (coherent within a group, balanced across warps when the batch's
// cost varies along it) and refills the lanes whose ray has finished (ballot + prefix) whenever fewer than kRefillBelow
// lanes are still tracing, so lanes do not idle while the warp's slowest ray finishes. One loop
// iteration advances every active lane by one step: one node (8 child boxes), one triangle, or one
// stack pop. Triangle work is postponed (its group pushed on the stack) while fewer than
// kPostponeBelow lanes of the warp have triangles and the lane still has nodes to visit (Ylitie,
// Karras and Laine, "Efficient incoherent ray traversal on GPUs through compressed wide BVHs",
// HPG 2017), so the warp mostly runs node steps or triangle steps together. Results are those of
// core::trace_ray: the closest hit does not depend on the visiting order (ties go to the lowest
// primitive index), the any-hit result is the occlusion bit.
// The counting variant (statistics for the roofline) runs the per-ray traversal of trace_core.h.
#include <algorithm>
#include <cuda_runtime.h>
#include <stdint.h>

#include "trace_core.h"
#include "trace_kernels.h"

namespace gbpt {
namespace {

constexpr int kThreads = 128;
constexpr int64_t kTopNodes = 1 + 8 + 64;  // staged nodes with top_levels: a full 8-wide tree's top three levels
constexpr unsigned kFull = 0xFFFFFFFFu;

// v-th ray of a warp: its (v / 32)-th group of 32 consecutive rays, the groups being dealt
// round-robin over the warps of the grid
__device__ __forceinline__ int64_t warp_ray(int64_t v, int64_t warp, int64_t n_warps)
{
    return ((v >> 5) * n_warps + warp) * 32 + (v & 31);
}

// refill_below: refill the warp when fewer lanes than this are tracing; postpone_below: run
// triangle steps only when at least this many lanes have them (else postpone)
// dynamic shared memory of the traversal kernels: SH stack entries per thread, entry-major
extern __shared__ uint2 trace_sh_stack[];

// The n_top nodes nearest the root (breadth-first order: the root, its children, theirs) copied
// from global memory into dynamic shared memory after the SH-deep stacks of the block, by all its
// threads; returns their shared copy (nullptr when n_top is 0). Every thread of the block must call
// it before any returns.
template <int SH>
__device__ __forceinline__ const uint4* stage_top_nodes(const uint4* __restrict__ nodes, uint32_t n_top)
{
    if (n_top == 0u) return nullptr;
    uint4* top = reinterpret_cast<uint4*>(trace_sh_stack + SH * blockDim.x);
    for (uint32_t i = threadIdx.x; i < 5u * n_top; i += blockDim.x) top[i] = __ldg(nodes + i);
    __syncthreads();
    return top;
}

template <bool ANY_HIT, int SH, int TRI, bool TOP>
__global__ void __launch_bounds__(256) trace_persistent(const uint4* __restrict__ nodes,
                                                             const float4* __restrict__ tris,
                                                             const float4* __restrict__ origin_tmin,
                                                             const float4* __restrict__ dir_tmax,
                                                             const int32_t* __restrict__ last_prim, int64_t n_rays,
                                                             int64_t rays_per_warp, int post_cap, int refill_below,
                                                             int postpone_below, float4* __restrict__ hits,
                                                             uint8_t* __restrict__ occluded, uint32_t n_top)
{
    const uint4* top = TOP ? stage_top_nodes<SH>(nodes, n_top) : nullptr;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int64_t next = 0;  // warp-uniform cursor over the warp's own rays
    const int64_t end = rays_per_warp;

    int64_t ray = -1;
    float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0, idx = 0, idy = 0, idz = 0, tmin = 0, tmax = 0;
    uint32_t oct_inv = 0;
    int32_t skip = -1;
    float t_best = 0, u_best = 0, v_best = 0;
    int32_t prim_best = -1;
    core::WatertightRay wr = {0, 1, 2, 0.0f, 0.0f, 0.0f};
    core::TraversalStack<SH> stack;
    uint2* const sh_col = trace_sh_stack + threadIdx.x;
    const int sh_stride = blockDim.x;
    int sp = 0, n_post = 0;
    uint2 ngroup = make_uint2(0u, 0u), tgroup = make_uint2(0u, 0u);

    for (;;)
    {
        // ---- refill idle lanes from the warp's chunk ----
        const unsigned idle = __ballot_sync(kFull, ray < 0);
        if (idle && next < end)
        {
            if (ray < 0)
            {
                const int64_t v = next + __popc(idle & ((1u << lane) - 1u));
                const int64_t r = warp_ray(v, warp, n_warps);
                if (v < end && r < n_rays)
                {
                    ray = r;
                    const float4 ot = origin_tmin[r], dt = dir_tmax[r];
                    ox = ot.x;
                    oy = ot.y;
                    oz = ot.z;
                    tmin = ot.w;
                    dx = dt.x;
                    dy = dt.y;
                    dz = dt.z;
                    tmax = dt.w;
                    idx = core::safe_rcp(dx);
                    idy = core::safe_rcp(dy);
                    idz = core::safe_rcp(dz);
                    oct_inv = (dx >= 0.0f ? 4u : 0u) | (dy >= 0.0f ? 2u : 0u) | (dz >= 0.0f ? 1u : 0u);
                    if constexpr (TRI == core::kTriWatertight) wr = core::watertight_ray(dx, dy, dz);
                    skip = last_prim ? last_prim[r] : -1;
                    t_best = tmax;
                    prim_best = -1;
                    sp = 0;
                    n_post = 0;
                    ngroup = make_uint2(0u, 0x80000000u);
                    tgroup = make_uint2(0u, 0u);
                }
            }
            next += __popc(idle);
        }
        if (__ballot_sync(kFull, ray >= 0) == 0u) break;

        // ---- traverse until the warp wants a refill ----
        for (;;)
        {
            const bool active = ray >= 0;
            const bool has_tri = active && tgroup.y != 0u;
            const bool has_node = active && (ngroup.y & 0xFF000000u) != 0u;
            const unsigned tri_lanes = __ballot_sync(kFull, has_tri);
            bool do_tri = has_tri && (!has_node || __popc(tri_lanes) >= postpone_below);
            if (has_tri && !do_tri)
            {
                if (n_post < post_cap)
                {
                    stack.push(sp, tgroup, sh_col, sh_stride);  // postponed triangle group (bits 24-31 clear)
                    n_post++;
                    tgroup.y = 0u;
                }
                else
                    do_tri = true;
            }
            bool finished = false;
            if (do_tri)
            {
                const int b = __ffs(tgroup.y) - 1;
                tgroup.y &= tgroup.y - 1u;
                const size_t ti = (size_t)(tgroup.x + (uint32_t)b);
                const float4 a = __ldg(tris + 3 * ti), b3 = __ldg(tris + 3 * ti + 1), c3 = __ldg(tris + 3 * ti + 2);
                float t, u, v;
                if (core::tri_test<TRI>(wr, a, b3, c3, ox, oy, oz, dx, dy, dz, t, u, v))
                {
                    const int32_t prim = __float_as_int(a.w);
                    if (t >= tmin && prim != skip)
                    {
                        if (ANY_HIT)
                        {
                            if (t < tmax)
                            {
                                prim_best = prim;
                                finished = true;
                            }
                        }
                        else if (t < t_best || (t == t_best && prim < prim_best))
                        {
                            t_best = t;
                            u_best = u;
                            v_best = v;
                            prim_best = prim;
                        }
                    }
                }
            }
            else if (has_node)
            {
                const uint32_t hits_imask = ngroup.y;
                const uint32_t bit = 31u - __clz(hits_imask & 0xFF000000u);
                ngroup.y &= ~(1u << bit);
                if (ngroup.y & 0xFF000000u) stack.push(sp, ngroup, sh_col, sh_stride);
                const uint32_t slot = (bit - 24u) ^ oct_inv;
                const uint32_t rel = __popc(hits_imask & ~(0xFFFFFFFFu << slot));
                const uint32_t ni = ngroup.x + rel;
                uint4 w0, w1, w2, w3, w4;
                if (TOP && ni < n_top)
                {
                    const uint4* tp = top + 5 * ni;
                    w0 = tp[0];
                    w1 = tp[1];
                    w2 = tp[2];
                    w3 = tp[3];
                    w4 = tp[4];
                }
                else
                {
                    const uint4* np = nodes + 5 * (size_t)ni;
                    w0 = __ldg(np + 0);
                    w1 = __ldg(np + 1);
                    w2 = __ldg(np + 2);
                    w3 = __ldg(np + 3);
                    w4 = __ldg(np + 4);
                }
                const uint32_t hm = core::intersect_children(w0, w1, w2, w3, w4, ox, oy, oz, idx, idy, idz, tmin,
                                                             ANY_HIT ? tmax : t_best, oct_inv);
                ngroup = make_uint2(w1.x, (hm & 0xFF000000u) | (w0.w >> 24));
                tgroup = make_uint2(w1.y, hm & 0x00FFFFFFu);
            }
            else if (active)
            {
                if (sp > 0)
                {
                    const uint2 g = stack.pop(sp, sh_col, sh_stride);
                    if (g.y & 0xFF000000u)
                        ngroup = g;
                    else
                    {
                        tgroup = g;
                        n_post--;
                    }
                }
                else
                    finished = true;
            }
            if (finished)
            {
                if (ANY_HIT)
                {
                    if (occluded) occluded[ray] = prim_best >= 0 ? 1 : 0;
                }
                else if (hits)
                    hits[ray] = prim_best >= 0 ? make_float4(t_best, u_best, v_best, __int_as_float(prim_best))
                                               : make_float4(-1.0f, 0.0f, 0.0f, __int_as_float(-1));
                ray = -1;
            }
            const unsigned act = __ballot_sync(kFull, ray >= 0);
            if (act == 0u || (__popc(act) < refill_below && next < end)) break;
        }
    }
}

// Per-lane fetch: the per-ray loop (a node, then all triangles of its hit leaves, then a pop), and
// a lane whose ray finished takes the next ray of its warp's chunk at once (a shared-memory
// counter per warp), so lanes do not wait for the warp's longest ray.
template <bool ANY_HIT, int SH, int TRI, bool TOP>
__global__ void __launch_bounds__(256) trace_fetch(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                                   const float4* __restrict__ origin_tmin,
                                                   const float4* __restrict__ dir_tmax,
                                                   const int32_t* __restrict__ last_prim, int64_t n_rays,
                                                   int64_t rays_per_warp, float4* __restrict__ hits,
                                                   uint8_t* __restrict__ occluded, uint32_t n_top)
{
    __shared__ unsigned int next_ray[8];  // per warp of the block (<= 256 threads)
    const uint4* top = TOP ? stage_top_nodes<SH>(nodes, n_top) : nullptr;
    const int wib = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) next_ray[wib] = 0u;
    __syncwarp();
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (;;)
    {
        const int64_t v = (int64_t)atomicAdd(&next_ray[wib], 1u);
        const int64_t ray = warp_ray(v, warp, n_warps);
        if (v >= rays_per_warp || ray >= n_rays) break;
        uint32_t cn = 0, ct = 0;
        const float4 h = core::trace_ray<ANY_HIT, false, SH, TRI, TOP>(nodes, tris, origin_tmin[ray], dir_tmax[ray],
                                                                       last_prim ? last_prim[ray] : -1, cn, ct,
                                                                       trace_sh_stack + threadIdx.x, blockDim.x, top,
                                                                       n_top);
        if (ANY_HIT)
        {
            if (occluded) occluded[ray] = __float_as_int(h.w) >= 0 ? 1 : 0;
        }
        else if (hits)
            hits[ray] = h;
    }
}

// per-ray traversal, one thread per ray; COUNT adds node / triangle counters (statistics)
template <bool ANY_HIT, bool COUNT, int SH, int TRI, bool TOP>
__global__ void __launch_bounds__(256) trace_ray_kernel(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                                               const float4* __restrict__ origin_tmin,
                                                               const float4* __restrict__ dir_tmax,
                                                               const int32_t* __restrict__ last_prim, int64_t n_rays,
                                                               float4* __restrict__ hits, uint8_t* __restrict__ occluded,
                                                               unsigned long long* __restrict__ counters, uint32_t n_top)
{
    const uint4* top = TOP ? stage_top_nodes<SH>(nodes, n_top) : nullptr;
    const int64_t ray = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ray >= n_rays) return;
    uint32_t n_nodes = 0, n_tris = 0;
    const float4 h = core::trace_ray<ANY_HIT, COUNT, SH, TRI, TOP>(nodes, tris, origin_tmin[ray], dir_tmax[ray],
                                                                   last_prim ? last_prim[ray] : -1, n_nodes, n_tris,
                                                                   trace_sh_stack + threadIdx.x, blockDim.x, top, n_top);
    if (ANY_HIT)
    {
        if (occluded) occluded[ray] = __float_as_int(h.w) >= 0 ? 1 : 0;
    }
    else if (hits)
        hits[ray] = h;
    if (!COUNT) return;
    const unsigned m = __activemask();
    const unsigned sn = __reduce_add_sync(m, n_nodes);
    const unsigned st = __reduce_add_sync(m, n_tris);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1))
    {
        atomicAdd(counters + 0, (unsigned long long)sn);
        atomicAdd(counters + 1, (unsigned long long)st);
    }
}

int sm_count()
{
    static int n = 0;
    if (n == 0)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace

TraceConfig default_trace_config(bool any_hit)
{
    TraceConfig c;
    c.kernel = any_hit ? kTraceKernelPerRay : kTraceKernelPersistent;
    c.block = 128;
    c.refill_below = 12;
    c.postpone_below = 8;
    c.blocks_per_sm = 8;
    c.shared_stack = 0;
    c.triangle_test = core::kTriMollerTrumbore;
    c.top_levels = 0;
    return c;
}

bool valid_trace_config(const TraceConfig& c)
{
    const bool block_ok = c.block == 32 || c.block == 64 || c.block == 128 || c.block == 256;
    return (c.kernel == kTraceKernelPerRay || c.kernel == kTraceKernelPersistent || c.kernel == kTraceKernelFetch) &&
           block_ok && c.refill_below >= 1 &&
           c.refill_below <= 32 && c.postpone_below >= 0 && c.postpone_below <= 32 && c.blocks_per_sm >= 1 &&
           c.blocks_per_sm <= 64 && (c.shared_stack == 0 || c.shared_stack == 8 || c.shared_stack == 16) &&
           (c.triangle_test == core::kTriMollerTrumbore || c.triangle_test == core::kTriWatertight) &&
           (c.top_levels == 0 || (c.top_levels == 1 && c.shared_stack == 0));
}

namespace {

// the launches of one shared-stack depth SH (dynamic shared memory: SH entries per thread)
template <int SH, int TRI, bool TOP>
cudaError_t launch_trace_sh(const DeviceBVH& bvh, const float* origin_tmin, const float* dir_tmax,
                            const int32_t* last_prim, int64_t n_rays, float* hits, uint8_t* occluded, bool any_hit,
                            unsigned long long* counters, cudaStream_t stream, const TraceConfig& cfg)
{
    const uint4* nodes = reinterpret_cast<const uint4*>(bvh.nodes);
    const float4* tris = reinterpret_cast<const float4*>(bvh.tris);
    const float4* o = reinterpret_cast<const float4*>(origin_tmin);
    const float4* d = reinterpret_cast<const float4*>(dir_tmax);
    float4* h = reinterpret_cast<float4*>(hits);
    // the nodes nearest the root staged in shared memory (top_levels): the root's three levels
    const uint32_t n_top = (TOP && !counters) ? (uint32_t)std::min<int64_t>(kTopNodes, bvh.n_nodes) : 0u;
    const size_t top_bytes = (size_t)n_top * 5 * sizeof(uint4);
    if (counters || cfg.kernel == kTraceKernelPerRay)
    {
        const int threads = counters ? kThreads : cfg.block;
        const int64_t blocks = (n_rays + threads - 1) / threads;
        const size_t smem = (size_t)SH * threads * sizeof(uint2) + top_bytes;
        if (counters)
        {
            if (any_hit)
                trace_ray_kernel<true, true, 0, TRI, false><<<(unsigned)blocks, threads, 0, stream>>>(nodes, tris, o, d, last_prim, n_rays,
                                                                                     h, occluded, counters, 0u);
            else
                trace_ray_kernel<false, true, 0, TRI, false><<<(unsigned)blocks, threads, 0, stream>>>(nodes, tris, o, d, last_prim,
                                                                                      n_rays, h, occluded, counters, 0u);
        }
        else if (any_hit)
            trace_ray_kernel<true, false, SH, TRI, TOP><<<(unsigned)blocks, threads, smem, stream>>>(nodes, tris, o, d, last_prim, n_rays,
                                                                                  h, occluded, nullptr, n_top);
        else
            trace_ray_kernel<false, false, SH, TRI, TOP><<<(unsigned)blocks, threads, smem, stream>>>(nodes, tris, o, d, last_prim, n_rays,
                                                                                   h, occluded, nullptr, n_top);
        return cudaGetLastError();
    }
    // persistent grids: blocks_per_sm blocks per SM, each warp owning a contiguous chunk of rays
    const int threads = cfg.block;
    const size_t smem = (size_t)SH * threads * sizeof(uint2) + top_bytes;
    if (cfg.kernel == kTraceKernelFetch)
    {
        const int64_t max_blocks = (int64_t)sm_count() * cfg.blocks_per_sm;
        const int64_t needed = (n_rays + threads - 1) / threads;
        const int64_t blocks = needed < max_blocks ? needed : max_blocks;
        const int64_t warps = blocks * (threads / 32);
        const int64_t per_warp = ((n_rays + 31) / 32 + warps - 1) / warps * 32;  // whole groups of 32
        if (any_hit)
            trace_fetch<true, SH, TRI, TOP><<<(unsigned)blocks, threads, smem, stream>>>(nodes, tris, o, d, last_prim, n_rays, per_warp, h,
                                                                        occluded, n_top);
        else
            trace_fetch<false, SH, TRI, TOP><<<(unsigned)blocks, threads, smem, stream>>>(nodes, tris, o, d, last_prim, n_rays, per_warp, h,
                                                                         occluded, n_top);
        return cudaGetLastError();
    }
    const int64_t max_blocks = (int64_t)sm_count() * cfg.blocks_per_sm;
    const int64_t needed = (n_rays + threads - 1) / threads;
    const int64_t blocks = needed < max_blocks ? needed : max_blocks;
    const int64_t warps = blocks * (threads / 32);
    const int64_t per_warp = ((n_rays + 31) / 32 + warps - 1) / warps * 32;  // whole groups of 32
    const int post_cap = kTraversalStack - bvh.depth - 1 > 0 ? kTraversalStack - bvh.depth - 1 : 0;
    if (any_hit)
        trace_persistent<true, SH, TRI, TOP><<<(unsigned)blocks, threads, smem, stream>>>(nodes, tris, o, d, last_prim, n_rays, per_warp,
                                                                         post_cap, cfg.refill_below, cfg.postpone_below, h,
                                                                         occluded, n_top);
    else
        trace_persistent<false, SH, TRI, TOP><<<(unsigned)blocks, threads, smem, stream>>>(nodes, tris, o, d, last_prim, n_rays, per_warp,
                                                                          post_cap, cfg.refill_below, cfg.postpone_below,
                                                                          h, occluded, n_top);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_trace(const DeviceBVH& bvh, const float* origin_tmin, const float* dir_tmax,
                         const int32_t* last_prim, int64_t n_rays, float* hits, uint8_t* occluded, bool any_hit,
                         unsigned long long* counters, cudaStream_t stream, const TraceConfig* cfg_in)
{
    if (n_rays <= 0) return cudaSuccess;
    const TraceConfig cfg = cfg_in ? *cfg_in : default_trace_config(any_hit);
    // the counting build traces with the parity triangle test (node and triangle counts); the top
    // levels in shared memory come with the local-memory stack only (shared_stack 0)
    if (cfg.triangle_test == core::kTriWatertight && !counters)
    {
        if (cfg.top_levels)
            return launch_trace_sh<0, core::kTriWatertight, true>(bvh, origin_tmin, dir_tmax, last_prim, n_rays, hits,
                                                                  occluded, any_hit, counters, stream, cfg);
        switch (cfg.shared_stack)
        {
        case 8: return launch_trace_sh<8, core::kTriWatertight, false>(bvh, origin_tmin, dir_tmax, last_prim, n_rays, hits,
                                                                       occluded, any_hit, counters, stream, cfg);
        case 16: return launch_trace_sh<16, core::kTriWatertight, false>(bvh, origin_tmin, dir_tmax, last_prim, n_rays,
                                                                         hits, occluded, any_hit, counters, stream, cfg);
        default: return launch_trace_sh<0, core::kTriWatertight, false>(bvh, origin_tmin, dir_tmax, last_prim, n_rays,
                                                                        hits, occluded, any_hit, counters, stream, cfg);
        }
    }
    if (cfg.top_levels && !counters)
        return launch_trace_sh<0, core::kTriMollerTrumbore, true>(bvh, origin_tmin, dir_tmax, last_prim, n_rays, hits,
                                                                  occluded, any_hit, counters, stream, cfg);
    switch (counters ? 0 : cfg.shared_stack)
    {
    case 8: return launch_trace_sh<8, core::kTriMollerTrumbore, false>(bvh, origin_tmin, dir_tmax, last_prim, n_rays, hits,
                                                                       occluded, any_hit, counters, stream, cfg);
    case 16: return launch_trace_sh<16, core::kTriMollerTrumbore, false>(bvh, origin_tmin, dir_tmax, last_prim, n_rays,
                                                                         hits, occluded, any_hit, counters, stream, cfg);
    default: return launch_trace_sh<0, core::kTriMollerTrumbore, false>(bvh, origin_tmin, dir_tmax, last_prim, n_rays,
                                                                        hits, occluded, any_hit, counters, stream, cfg);
    }
}

}  // namespace gbpt
