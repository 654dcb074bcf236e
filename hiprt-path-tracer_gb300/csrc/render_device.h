// Device helpers shared by the path-tracing kernels (render.cu) and the ReSTIR DI kernels
// (restir.cu): warp-aggregated queue appends, the Lambertian BSDF, the backface fix of hit
// normals, emissive-triangle light sampling, and the seeding of BSDF samples.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "principled.h"
#include "render_common.h"
#include "render_kernels.h"

namespace gbpt {

// Appends one entry per calling thread with 'want' set; returns the slot index (or -1).
// Warp-aggregated: one atomicAdd per warp (ballot + popc prefix).
__device__ __forceinline__ int warp_append(int32_t* counter, bool want)
{
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, want);
    if (!want) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void warp_count(unsigned long long* counter, bool c)
{
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, c);
    if ((threadIdx.x & 31) == __ffs(active) - 1 && mask) atomicAdd(counter, (unsigned long long)__popc(mask));
}

__device__ __forceinline__ void store_rng(uint64_t* p, const Pcg32& r) { *p = r.state; }

// ---------------------------------------------------------------------------------------------
// Lambertian BSDF (src/Device/includes/BSDFs/Lambertian.h:14-58)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ V3 lambert_eval(V3 albedo, float NoL, float& pdf)
{
    pdf = 0.0f;
    if (NoL <= 0.0f) return v3(0.0f, 0.0f, 0.0f);
    pdf = NoL * kInvPi;
    return albedo * kInvPi;
}

// fix_backfacing_normals (src/Device/includes/Intersect.h:142-176)
__device__ __forceinline__ void fix_backfacing(V3 view, V3& ng, V3& ns)
{
    if (dot(view, ng) < 0.0f)
    {
        ng = -ng;
        ns = -ns;
    }
    if (dot(view, ns) < 0.0f) ns = -ns;
    V3 refl = 2.0f * dot(view, ns) * ns - view;
    if (dot(refl, ng) <= 0.0f)
    {
        refl = refl - normalize((dot(refl, ng) - 0.01f) * ng);
        ns = normalize(view + refl);
    }
}

// ---------------------------------------------------------------------------------------------
// light sample on an emissive triangle (sample_one_emissive_triangle_uniform / _power,
// src/Device/includes/LightSampling/LightUtils.h:248-309; Heitz 2019 point, :150-199)
// ---------------------------------------------------------------------------------------------
struct LightSample
{
    V3 point, normal, emission;
    float pdf_area;
    int triangle;
};

__device__ __forceinline__ LightSample sample_light(const SceneView& s, const RenderConst& rc, Pcg32& rng)
{
    int e;
    if (rc.light_sampling == GBPT_LIGHT_POWER)
    {
        e = rng.index(s.n_emissive);
        if (rng.next() > __ldg(s.alias_prob + e)) e = __ldg(s.alias_index + e);
    }
    else
        e = rng.index(s.n_emissive);
    const int lt = __ldg(s.emissive + e);
    float r1 = rng.next(), r2 = rng.next();
    square_to_triangle(r1, r2);
    V3 la, lb, lc;
    load_triangle(s, lt, la, lb, lc);
    const V3 ab = lb - la, ac = lc - la;
    const V3 nrm = cross(ab, ac);
    const float len = length(nrm);
    LightSample ls;
    ls.triangle = lt;
    ls.point = la + ab * r1 + ac * r2;
    ls.normal = nrm / len;
    const float area = 0.5f * len;
    ls.emission = xyz(s.materials[__ldg(s.material_of + lt)].emission);
    ls.pdf_area = 1.0f / area;
    if (rc.light_sampling == GBPT_LIGHT_POWER)
        ls.pdf_area *= (luminance(ls.emission) * area) / s.power_sum;
    else
        ls.pdf_area /= (float)s.n_emissive;
    return ls;
}

// A BSDF sample draws its random numbers from a Xorshift32 generator (the reference's generator,
// src/HostDeviceCommon/Xorshift.h) seeded by the path's PCG stream, so the same numbers can be
// replayed through the reference's own BSDF.
__device__ __forceinline__ bsdf::Xorshift32 bsdf_rng(Pcg32& rng)
{
    uint32_t seed = rng.next_u32();
    return bsdf::Xorshift32{seed != 0u ? seed : 0x9E3779B9u};
}

// MaterialUtils::can_do_light_sampling (MaterialUtils.h:71-93): a material whose every lobe is a
// delta distribution skips light sampling (and its random numbers).
__device__ __forceinline__ bool can_light_sample(const bsdf::Material& m)
{
    const bool smooth_base = bsdf::is_smooth(m.roughness) && (m.metallic == 1.0f || m.transmission == 1.0f);
    const bool smooth_coat = m.coat == 0.0f || bsdf::is_smooth(m.coat_roughness);
    const bool smooth_second = bsdf::is_smooth(m.second_roughness) || m.second_weight == 0.0f;
    return !(smooth_base && smooth_coat && smooth_second);
}

// Guided sampling applies to materials whose BSDF has no delta lobe and no transmission: every
// lobe then has a density that the one-sample MIS with the learned mixture can use.
__device__ __forceinline__ bool guidable(const bsdf::Material& m)
{
    if (m.transmission > 0.0f || m.diffuse_transmission > 0.0f) return false;
    if (bsdf::is_smooth(m.roughness) && (m.metallic > 0.0f || m.specular > 0.0f)) return false;
    if (m.coat > 0.0f && bsdf::is_smooth(m.coat_roughness)) return false;
    if (m.metallic > 0.0f && m.second_weight > 0.0f && bsdf::is_smooth(m.second_roughness)) return false;
    return true;
}

// Hash deciding which path vertices become guiding training records (independent of the path's
// random numbers, so recording never changes the rendered image)
__device__ __forceinline__ uint32_t record_hash(uint32_t slot, uint32_t bounce, uint32_t frame)
{
    uint32_t h = slot * 0x9E3779B1u ^ (bounce * 0x85EBCA77u + frame * 0xC2B2AE3Du + 0x27D4EB2Fu);
    h ^= h >> 16;
    h *= 0x7FEB352Du;
    h ^= h >> 15;
    h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h;
}

}  // namespace gbpt
