// C ABI of libgbpt: handles, status codes, argument checks and launches (declared in include/gbpt.h).
//
// Replaces the reference's host-side launch layer for the intersection path: HIPRTGeometry
// (src/HIPRT-Orochi/HIPRTScene.h:87-202) and the traversal calls made from
// src/Device/includes/Intersect.h. Every failure is returned as a gbpt_status with a
// thread-local message; nothing exits, aborts or traps.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/gbpt.h"
#include "bvh.h"
#include "handles.h"
#include "trace_kernels.h"

namespace {
thread_local std::string g_last_error;
}

namespace gbpt {
gbpt_status set_error(gbpt_status s, const std::string& msg)
{
    g_last_error = msg;
    return s;
}

gbpt_status cuda_error(cudaError_t e, const char* what)
{
    gbpt_status s = (e == cudaErrorMemoryAllocation) ? GBPT_ERROR_OOM : GBPT_ERROR_CUDA;
    return set_error(s, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}
}  // namespace gbpt

namespace {

gbpt_status fail(gbpt_status s, const std::string& msg) { return gbpt::set_error(s, msg); }
gbpt_status cuda_fail(cudaError_t e, const char* what) { return gbpt::cuda_error(e, what); }

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

gbpt_status check_rays(const gbpt_bvh* bvh, const float* o, const float* d, int64_t n)
{
    if (!bvh) return fail(GBPT_ERROR_INVALID_ARG, "bvh is NULL");
    if (n < 0) return fail(GBPT_ERROR_INVALID_ARG, "n_rays is negative");
    if (n > 0 && (!o || !d)) return fail(GBPT_ERROR_INVALID_ARG, "ray buffers are NULL");
    if (!aligned16(o) || !aligned16(d)) return fail(GBPT_ERROR_INVALID_ARG, "ray buffers must be 16-byte aligned");
    if (n > (int64_t)0x7FFFFFFF * 128) return fail(GBPT_ERROR_INVALID_ARG, "n_rays too large for one launch");
    return GBPT_OK;
}

}  // namespace

extern "C" {

const char* gbpt_status_string(gbpt_status s)
{
    switch (s)
    {
    case GBPT_OK: return "ok";
    case GBPT_ERROR_INVALID_ARG: return "invalid argument";
    case GBPT_ERROR_OOM: return "out of memory";
    case GBPT_ERROR_CUDA: return "CUDA error";
    case GBPT_ERROR_TIMEOUT: return "timeout";
    case GBPT_ERROR_NAN: return "NaN detected";
    case GBPT_ERROR_UNSUPPORTED: return "unsupported";
    case GBPT_ERROR_BVH_TOO_DEEP: return "BVH too deep";
    }
    return "unknown status";
}

const char* gbpt_last_error(void) { return g_last_error.c_str(); }

int32_t gbpt_version(void) { return 1; }

gbpt_status gbpt_bvh_build(const int32_t* indices, const float* positions, int64_t n_vertices, int64_t n_triangles,
                           const gbpt_bvh_params* params, gbpt_bvh** out)
{
    if (!out) return fail(GBPT_ERROR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (n_triangles < 0 || n_vertices < 0) return fail(GBPT_ERROR_INVALID_ARG, "negative sizes");
    if (n_triangles > 0 && (!indices || !positions)) return fail(GBPT_ERROR_INVALID_ARG, "geometry buffers are NULL");

    gbpt::BuildParams bp;
    if (params)
    {
        if (params->sah_bins) bp.sah_bins = params->sah_bins;
        if (params->max_leaf_size) bp.max_leaf = params->max_leaf_size;
        bp.threads = params->num_threads;
    }
    gbpt::HostBVH host;
    bool too_deep = false;
    std::string err;
    try
    {
        err = gbpt::build_wide_bvh(indices, positions, n_vertices, n_triangles, bp, host, too_deep);
    }
    catch (const std::bad_alloc&)
    {
        return fail(GBPT_ERROR_OOM, "host allocation failed during the BVH build");
    }
    if (!err.empty()) return fail(too_deep ? GBPT_ERROR_BVH_TOO_DEEP : GBPT_ERROR_INVALID_ARG, err);

    auto t0 = std::chrono::steady_clock::now();
    gbpt_bvh* b = new (std::nothrow) gbpt_bvh();
    if (!b) return fail(GBPT_ERROR_OOM, "host allocation failed");
    cudaGetDevice(&b->device);
    const size_t node_bytes = host.nodes.size() * sizeof(gbpt::WideNode);
    const size_t tri_bytes = std::max<size_t>(16, host.tris.size() * sizeof(float));
    void* dn = nullptr;
    void* dt = nullptr;
    cudaError_t e = cudaMalloc(&dn, node_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&dt, tri_bytes);
    if (e == cudaSuccess) e = cudaMemcpy(dn, host.nodes.data(), node_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !host.tris.empty())
        e = cudaMemcpy(dt, host.tris.data(), host.tris.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        cudaFree(dn);
        cudaFree(dt);
        delete b;
        return cuda_fail(e, "BVH upload");
    }
    b->dev.nodes = dn;
    b->dev.tris = dt;
    b->dev.n_nodes = (int64_t)host.nodes.size();
    b->dev.n_tris = (int64_t)(host.tris.size() / 12);
    b->dev.depth = host.wide_depth;
    std::memset(&b->stats, 0, sizeof(b->stats));
    b->stats.n_triangles = n_triangles;
    b->stats.n_bvh_triangles = b->dev.n_tris;
    b->stats.n_nodes = b->dev.n_nodes;
    b->stats.n_binary_nodes = host.n_binary_nodes;
    b->stats.wide_depth = host.wide_depth;
    b->stats.node_bytes = (int32_t)sizeof(gbpt::WideNode);
    b->stats.triangle_bytes = 48;
    b->stats.device_bytes = (int64_t)(node_bytes + tri_bytes);
    b->stats.build_seconds = host.build_seconds;
    b->stats.upload_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = b;
    return GBPT_OK;
}

gbpt_status gbpt_bvh_get_stats(const gbpt_bvh* bvh, gbpt_bvh_stats* out)
{
    if (!bvh || !out) return fail(GBPT_ERROR_INVALID_ARG, "NULL argument");
    *out = bvh->stats;
    return GBPT_OK;
}

gbpt_status gbpt_bvh_destroy(gbpt_bvh* bvh)
{
    if (!bvh) return GBPT_OK;
    HostTraceStaging& h = bvh->staging;
    if (h.buf) cudaFree(h.buf);
    if (h.side) cudaStreamDestroy(h.side);
    if (h.start) cudaEventDestroy(h.start);
    if (h.side_done) cudaEventDestroy(h.side_done);
    cudaError_t e1 = cudaFree(const_cast<void*>(bvh->dev.nodes));
    cudaError_t e2 = cudaFree(const_cast<void*>(bvh->dev.tris));
    delete bvh;
    if (e1 != cudaSuccess) return cuda_fail(e1, "BVH free");
    if (e2 != cudaSuccess) return cuda_fail(e2, "BVH free");
    return GBPT_OK;
}

gbpt_status gbpt_trace_closest(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                               const int32_t* last_prim, int64_t n_rays, float* hits, void* stream)
{
    gbpt_status s = check_rays(bvh, origin_tmin, dir_tmax, n_rays);
    if (s != GBPT_OK) return s;
    if (n_rays > 0 && !hits) return fail(GBPT_ERROR_INVALID_ARG, "hits is NULL");
    if (!aligned16(hits)) return fail(GBPT_ERROR_INVALID_ARG, "hits must be 16-byte aligned");
    cudaError_t e = gbpt::launch_trace(bvh->dev, origin_tmin, dir_tmax, last_prim, n_rays, hits, nullptr, false, nullptr,
                                       (cudaStream_t)stream, &bvh->cfg[0]);
    return e == cudaSuccess ? GBPT_OK : cuda_fail(e, "closest-hit launch");
}

gbpt_status gbpt_trace_any(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                           const int32_t* last_prim, int64_t n_rays, uint8_t* occluded, void* stream)
{
    gbpt_status s = check_rays(bvh, origin_tmin, dir_tmax, n_rays);
    if (s != GBPT_OK) return s;
    if (n_rays > 0 && !occluded) return fail(GBPT_ERROR_INVALID_ARG, "occluded is NULL");
    cudaError_t e = gbpt::launch_trace(bvh->dev, origin_tmin, dir_tmax, last_prim, n_rays, nullptr, occluded, true,
                                       nullptr, (cudaStream_t)stream, &bvh->cfg[1]);
    return e == cudaSuccess ? GBPT_OK : cuda_fail(e, "any-hit launch");
}

gbpt_status gbpt_trace_count(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                             const int32_t* last_prim, int64_t n_rays, int32_t any_hit, unsigned long long* counters,
                             void* stream)
{
    gbpt_status s = check_rays(bvh, origin_tmin, dir_tmax, n_rays);
    if (s != GBPT_OK) return s;
    if (!counters) return fail(GBPT_ERROR_INVALID_ARG, "counters is NULL");
    cudaError_t e = gbpt::launch_trace(bvh->dev, origin_tmin, dir_tmax, last_prim, n_rays, nullptr, nullptr, any_hit != 0,
                                       counters, (cudaStream_t)stream);
    return e == cudaSuccess ? GBPT_OK : cuda_fail(e, "counting launch");
}

// Host-buffer trace: the batch is cut into chunks issued alternately on the caller's stream and a
// side stream; each chunk copies its rays in, traces and copies its results out, so that one
// chunk's copies overlap the other stream's traversal (the copy engines run beside the SMs; with
// pinned host buffers the copies are asynchronous). The device staging is kept with the BVH and
// reused. Results do not depend on the chunking: every ray is traced on its own.
static gbpt_status trace_host(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                              const int32_t* last_prim, int64_t n, void* out, bool any_hit, cudaStream_t st)
{
    gbpt_status s = check_rays(bvh, origin_tmin, dir_tmax, n);
    if (s != GBPT_OK) return s;
    if (n > 0 && !out) return fail(GBPT_ERROR_INVALID_ARG, "output is NULL");
    if (n == 0) return GBPT_OK;
    const size_t ray_bytes = (size_t)n * 16;
    const size_t out_stride = any_hit ? 1 : 16;
    const size_t lp_off = 2 * ray_bytes;
    const size_t out_off = lp_off + (((size_t)n * 4 + 255) & ~(size_t)255);
    const size_t need = out_off + (size_t)n * out_stride;

    HostTraceStaging& h = bvh->staging;
    std::lock_guard<std::mutex> lock(h.mu);
    cudaError_t e = cudaSuccess;
    if (!h.side) e = cudaStreamCreateWithFlags(&h.side, cudaStreamNonBlocking);
    if (e == cudaSuccess && !h.start) e = cudaEventCreateWithFlags(&h.start, cudaEventDisableTiming);
    if (e == cudaSuccess && !h.side_done) e = cudaEventCreateWithFlags(&h.side_done, cudaEventDisableTiming);
    if (e == cudaSuccess && h.cap < need)
    {
        // the previous staging may still be read by work queued on the caller's stream
        if (h.buf) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess && h.buf) e = cudaFree(h.buf);
        h.buf = nullptr;
        h.cap = 0;
        if (e == cudaSuccess) e = cudaMalloc((void**)&h.buf, need);
        if (e == cudaSuccess) h.cap = need;
    }
    if (e != cudaSuccess) return cuda_fail(e, "host-buffer trace staging");
    float* d_o = (float*)h.buf;
    float* d_d = (float*)(h.buf + ray_bytes);
    int32_t* d_lp = last_prim ? (int32_t*)(h.buf + lp_off) : nullptr;
    char* d_out = h.buf + out_off;

    // the side stream starts after the caller's earlier work
    e = cudaEventRecord(h.start, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h.side, h.start, 0);
    const int64_t chunk = std::max<int64_t>((int64_t)1 << 20, (n + 7) / 8);
    int c = 0;
    for (int64_t b = 0; e == cudaSuccess && b < n; b += chunk, c++)
    {
        const int64_t m = std::min(chunk, n - b);
        cudaStream_t cs = (c & 1) ? h.side : st;
        e = cudaMemcpyAsync(d_o + 4 * b, origin_tmin + 4 * b, (size_t)m * 16, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_d + 4 * b, dir_tmax + 4 * b, (size_t)m * 16, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess && d_lp)
            e = cudaMemcpyAsync(d_lp + b, last_prim + b, (size_t)m * 4, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess)
            e = gbpt::launch_trace(bvh->dev, d_o + 4 * b, d_d + 4 * b, d_lp ? d_lp + b : nullptr, m,
                                   any_hit ? nullptr : (float*)(d_out + b * 16),
                                   any_hit ? (uint8_t*)(d_out + b) : nullptr, any_hit, nullptr, cs,
                                   &bvh->cfg[any_hit ? 1 : 0]);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync((char*)out + b * out_stride, d_out + b * out_stride, (size_t)m * out_stride,
                                cudaMemcpyDeviceToHost, cs);
    }
    // the caller's stream ends after the side stream's chunks
    cudaError_t er = cudaEventRecord(h.side_done, h.side);
    if (er == cudaSuccess) er = cudaStreamWaitEvent(st, h.side_done, 0);
    if (e == cudaSuccess) e = er;
    cudaError_t es = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = es;
    return e == cudaSuccess ? GBPT_OK : cuda_fail(e, "host-buffer trace");
}

gbpt_status gbpt_trace_closest_host(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                    const int32_t* last_prim, int64_t n_rays, float* hits, void* stream)
{
    return trace_host(bvh, origin_tmin, dir_tmax, last_prim, n_rays, hits, false, (cudaStream_t)stream);
}

gbpt_status gbpt_trace_any_host(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                const int32_t* last_prim, int64_t n_rays, uint8_t* occluded, void* stream)
{
    return trace_host(bvh, origin_tmin, dir_tmax, last_prim, n_rays, occluded, true, (cudaStream_t)stream);
}

namespace {

gbpt::TraceConfig from_c(const gbpt_trace_config& c)
{
    gbpt::TraceConfig t;
    t.kernel = c.kernel;
    t.block = c.block;
    t.refill_below = c.refill_below;
    t.postpone_below = c.postpone_below;
    t.blocks_per_sm = c.blocks_per_sm;
    t.shared_stack = c.shared_stack;
    t.triangle_test = c.triangle_test;
    t.top_levels = c.top_levels;
    return t;
}

gbpt_trace_config to_c(const gbpt::TraceConfig& t)
{
    gbpt_trace_config c;
    std::memset(&c, 0, sizeof(c));
    c.kernel = t.kernel;
    c.block = t.block;
    c.refill_below = t.refill_below;
    c.postpone_below = t.postpone_below;
    c.blocks_per_sm = t.blocks_per_sm;
    c.shared_stack = t.shared_stack;
    c.triangle_test = t.triangle_test;
    c.top_levels = t.top_levels;
    return c;
}

}  // namespace

gbpt_status gbpt_bvh_set_trace_config(gbpt_bvh* bvh, int32_t any_hit, const gbpt_trace_config* cfg)
{
    if (!bvh || !cfg) return fail(GBPT_ERROR_INVALID_ARG, "NULL argument");
    const gbpt::TraceConfig t = from_c(*cfg);
    if (!gbpt::valid_trace_config(t)) return fail(GBPT_ERROR_INVALID_ARG, "invalid trace configuration");
    bvh->cfg[any_hit ? 1 : 0] = t;
    return GBPT_OK;
}

gbpt_status gbpt_bvh_get_trace_config(const gbpt_bvh* bvh, int32_t any_hit, gbpt_trace_config* cfg)
{
    if (!bvh || !cfg) return fail(GBPT_ERROR_INVALID_ARG, "NULL argument");
    *cfg = to_c(bvh->cfg[any_hit ? 1 : 0]);
    return GBPT_OK;
}

gbpt_status gbpt_trace_closest_cfg(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                   const int32_t* last_prim, int64_t n_rays, float* hits, const gbpt_trace_config* cfg,
                                   void* stream)
{
    gbpt_status s = check_rays(bvh, origin_tmin, dir_tmax, n_rays);
    if (s != GBPT_OK) return s;
    if (n_rays > 0 && !hits) return fail(GBPT_ERROR_INVALID_ARG, "hits is NULL");
    if (!aligned16(hits)) return fail(GBPT_ERROR_INVALID_ARG, "hits must be 16-byte aligned");
    const gbpt::TraceConfig t = cfg ? from_c(*cfg) : bvh->cfg[0];
    if (!gbpt::valid_trace_config(t)) return fail(GBPT_ERROR_INVALID_ARG, "invalid trace configuration");
    cudaError_t e = gbpt::launch_trace(bvh->dev, origin_tmin, dir_tmax, last_prim, n_rays, hits, nullptr, false, nullptr,
                                       (cudaStream_t)stream, &t);
    return e == cudaSuccess ? GBPT_OK : cuda_fail(e, "closest-hit launch");
}

gbpt_status gbpt_trace_any_cfg(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                               const int32_t* last_prim, int64_t n_rays, uint8_t* occluded, const gbpt_trace_config* cfg,
                               void* stream)
{
    gbpt_status s = check_rays(bvh, origin_tmin, dir_tmax, n_rays);
    if (s != GBPT_OK) return s;
    if (n_rays > 0 && !occluded) return fail(GBPT_ERROR_INVALID_ARG, "occluded is NULL");
    const gbpt::TraceConfig t = cfg ? from_c(*cfg) : bvh->cfg[1];
    if (!gbpt::valid_trace_config(t)) return fail(GBPT_ERROR_INVALID_ARG, "invalid trace configuration");
    cudaError_t e = gbpt::launch_trace(bvh->dev, origin_tmin, dir_tmax, last_prim, n_rays, nullptr, occluded, true,
                                       nullptr, (cudaStream_t)stream, &t);
    return e == cudaSuccess ? GBPT_OK : cuda_fail(e, "any-hit launch");
}

gbpt_status gbpt_trace_autotune(gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax, const int32_t* last_prim,
                                int64_t n_rays, int32_t any_hit, int32_t store, gbpt_trace_config* best_out,
                                float* best_ms_out, void* stream)
{
    gbpt_status s = check_rays(bvh, origin_tmin, dir_tmax, n_rays);
    if (s != GBPT_OK) return s;
    if (n_rays <= 0) return fail(GBPT_ERROR_INVALID_ARG, "autotuning needs rays");
    cudaStream_t st = (cudaStream_t)stream;
    const bool ah = any_hit != 0;
    void* out = nullptr;
    cudaError_t e = cudaMallocAsync(&out, (size_t)n_rays * (ah ? 1 : 16), st);
    if (e != cudaSuccess) return cuda_fail(e, "autotune scratch");
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    // time per launch: the faster of two runs (the first also warms the caches)
    auto timed = [&](const gbpt::TraceConfig& c, float& ms) -> cudaError_t {
        ms = 1e30f;
        for (int rep = 0; rep < 2; rep++)
        {
            cudaError_t err = cudaEventRecord(ev0, st);
            if (err == cudaSuccess)
                err = gbpt::launch_trace(bvh->dev, origin_tmin, dir_tmax, last_prim, n_rays, ah ? nullptr : (float*)out,
                                         ah ? (uint8_t*)out : nullptr, ah, nullptr, st, &c);
            if (err == cudaSuccess) err = cudaEventRecord(ev1, st);
            if (err == cudaSuccess) err = cudaEventSynchronize(ev1);
            float t = 0.0f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&t, ev0, ev1);
            if (err != cudaSuccess) return err;
            ms = std::min(ms, t);
        }
        return cudaSuccess;
    };
    gbpt::TraceConfig best = bvh->cfg[ah ? 1 : 0];
    float best_ms = 0.0f;
    e = timed(best, best_ms);
    const int kernels[] = {gbpt::kTraceKernelPerRay, gbpt::kTraceKernelPersistent, gbpt::kTraceKernelFetch};
    const int blocks[] = {64, 128, 256};
    const int refills[] = {4, 8, 12, 16, 20, 24};
    const int postpones[] = {0, 4, 8, 12, 16, 24};
    const int per_sm[] = {2, 4, 8, 12, 16};
    const int shared[] = {0, 8, 16};
    const int binary[] = {0, 1};
    for (int pass = 0; pass < 2 && e == cudaSuccess; pass++)
    {
        // coordinates: kernel, block, shared-stack depth, top levels in shared memory, refill,
        // postpone, blocks per SM
        for (int coord = 0; coord < 7 && e == cudaSuccess; coord++)
        {
            if (best.kernel == gbpt::kTraceKernelPerRay && coord >= 4) break;
            if (best.kernel == gbpt::kTraceKernelFetch && (coord == 4 || coord == 5)) continue;
            const int* vals = coord == 0 ? kernels : coord == 1 ? blocks : coord == 2 ? shared
                            : coord == 3 ? binary : coord == 4 ? refills : coord == 5 ? postpones : per_sm;
            const int nv = coord <= 2 ? 3 : coord == 3 ? 2 : coord == 6 ? 5 : 6;
            for (int k = 0; k < nv && e == cudaSuccess; k++)
            {
                gbpt::TraceConfig c = best;
                int* field = coord == 0 ? &c.kernel : coord == 1 ? &c.block : coord == 2 ? &c.shared_stack
                           : coord == 3 ? &c.top_levels : coord == 4 ? &c.refill_below
                           : coord == 5 ? &c.postpone_below : &c.blocks_per_sm;
                if (*field == vals[k]) continue;
                *field = vals[k];
                // the top levels in shared memory come with the local-memory stack only
                if (c.top_levels && c.shared_stack != 0)
                {
                    if (coord == 2)
                        c.top_levels = 0;
                    else
                        c.shared_stack = 0;
                }
                float ms = 0.0f;
                e = timed(c, ms);
                if (e == cudaSuccess && ms < best_ms)
                {
                    best = c;
                    best_ms = ms;
                }
            }
        }
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaError_t ef = cudaFreeAsync(out, st);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "autotune");
    if (store) bvh->cfg[ah ? 1 : 0] = best;
    if (best_out) *best_out = to_c(best);
    if (best_ms_out) *best_ms_out = best_ms;
    return GBPT_OK;
}

}  // extern "C"
