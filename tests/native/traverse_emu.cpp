// TEST INFRASTRUCTURE ONLY — host build of the BVH builder and the shared traversal core
// (hiprt-path-tracer_gb300/csrc/bvh_build.cpp, trace_core.h) so that CPU-only test runs can check
// the 8-wide layout and the traversal logic against the oracle before any GPU run. The GPU tests
// then check that the CUDA kernels return the same bits. Built by tests/native/build_emu.py with
// -ffp-contract=off; never linked into libgbpt.
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "bvh.h"
#include "trace_core.h"

namespace {
struct Emu
{
    gbpt::HostBVH bvh;
    std::string err;
};
thread_local std::string g_err;
}

extern "C" {

const char* emu_last_error() { return g_err.c_str(); }

void* emu_build(const int32_t* indices, const float* positions, int64_t nv, int64_t nt, int max_leaf, int bins)
{
    Emu* e = new Emu();
    gbpt::BuildParams p;
    p.max_leaf = max_leaf;
    p.sah_bins = bins;
    bool too_deep = false;
    g_err = gbpt::build_wide_bvh(indices, positions, nv, nt, p, e->bvh, too_deep);
    if (!g_err.empty())
    {
        delete e;
        return nullptr;
    }
    return e;
}

void emu_free(void* h) { delete static_cast<Emu*>(h); }

/* out: n_nodes, n_stored_tris, wide_depth, n_binary_nodes */
void emu_stats(void* h, int64_t* out)
{
    Emu* e = static_cast<Emu*>(h);
    out[0] = (int64_t)e->bvh.nodes.size();
    out[1] = (int64_t)(e->bvh.tris.size() / 12);
    out[2] = e->bvh.wide_depth;
    out[3] = e->bvh.n_binary_nodes;
}

/* Copies the raw arrays: nodes (80 B each) and triangle records (48 B each). */
void emu_export(void* h, void* nodes, void* tris)
{
    Emu* e = static_cast<Emu*>(h);
    std::memcpy(nodes, e->bvh.nodes.data(), e->bvh.nodes.size() * sizeof(gbpt::WideNode));
    std::memcpy(tris, e->bvh.tris.data(), e->bvh.tris.size() * sizeof(float));
}

/* any_hit bit 0: any-hit traversal; bit 1: the watertight triangle test (else Moller-Trumbore) */
void emu_trace(void* h, const float* origin_tmin, const float* dir_tmax, const int32_t* last_prim, int64_t n, int any_hit,
               float* hits, int64_t* counters)
{
    const bool wt = (any_hit & 2) != 0;
    any_hit &= 1;
    Emu* e = static_cast<Emu*>(h);
    const uint4* nodes = reinterpret_cast<const uint4*>(e->bvh.nodes.data());
    const float4* tris = reinterpret_cast<const float4*>(e->bvh.tris.data());
    int64_t cn = 0, ct = 0;
    for (int64_t i = 0; i < n; i++)
    {
        float4 ot{origin_tmin[4 * i], origin_tmin[4 * i + 1], origin_tmin[4 * i + 2], origin_tmin[4 * i + 3]};
        float4 dt{dir_tmax[4 * i], dir_tmax[4 * i + 1], dir_tmax[4 * i + 2], dir_tmax[4 * i + 3]};
        int32_t lp = last_prim ? last_prim[i] : -1;
        uint32_t nn = 0, nt = 0;
        float4 r;
        if (wt)
            r = any_hit ? gbpt::core::trace_ray<true, true, 0, gbpt::core::kTriWatertight>(nodes, tris, ot, dt, lp, nn, nt)
                        : gbpt::core::trace_ray<false, true, 0, gbpt::core::kTriWatertight>(nodes, tris, ot, dt, lp, nn, nt);
        else
            r = any_hit ? gbpt::core::trace_ray<true, true>(nodes, tris, ot, dt, lp, nn, nt)
                        : gbpt::core::trace_ray<false, true>(nodes, tris, ot, dt, lp, nn, nt);
        cn += nn;
        ct += nt;
        std::memcpy(hits + 4 * i, &r, 16);
    }
    if (counters)
    {
        counters[0] += cn;
        counters[1] += ct;
    }
}

}  // extern "C"
