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

// A path's generator from its stored state: the PCG stream of the render seed, or under
// GBPT_RNG_REFERENCE the reference's Xorshift32 (inc = 0).
__device__ __forceinline__ Pcg32 load_rng(const RenderConst& rc, uint64_t state)
{
    Pcg32 r;
    r.state = state;
    r.inc = rc.rng_mode == GBPT_RNG_REFERENCE ? 0ULL : pcg_inc(rc.seed);
    return r;
}

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

// Solid-angle pdf with which light sampling would have chosen the point at distance 'dist' on
// emissive triangle 'prim' (emission Le, one-sided: 0 seen from behind) along unit direction wi
// (pdf_of_emissive_triangle_hit_area_measure, LightUtils.h:52-77, to solid angle,
// PDFConversion.h:19-38); 0 when the triangle is not seen from its front
__device__ __forceinline__ float emitter_hit_pdf(const SceneView& s, const RenderConst& rc, int prim, V3 Le, float dist,
                                                 V3 wi)
{
    V3 a, b, c;
    load_triangle(s, prim, a, b, c);
    const V3 nrm = cross(b - a, c - a);
    const float len = length(nrm);
    const float cos_l = fmaxf(0.0f, dot(nrm / len, -wi));
    if (!(cos_l > 0.0f)) return 0.0f;
    const float area = 0.5f * len;
    float pdf_area = 1.0f / area;
    if (rc.light_sampling == GBPT_LIGHT_POWER)
        pdf_area *= (luminance(Le) * area) / s.power_sum;
    else
        pdf_area /= (float)s.n_emissive;
    return area_to_solid_angle_pdf(pdf_area, dist, cos_l);
}

// Balance heuristic with sample counts as the reference writes it (Sampling.h:103-116): the count
// of technique a is left out of the numerator because RIS divides it out again.
__device__ __forceinline__ float balance_counts(float pdf_a, float n_a, float pdf_b, float n_b)
{
    return pdf_a == 0.0f ? 0.0f : pdf_a / (n_a * pdf_a + n_b * pdf_b);
}

// The light candidates of RIS direct lighting (sample_bsdf_and_lights_RIS_reservoir,
// src/Device/includes/RIS/RIS.h:96-198): M light samples, target p^ = luminance(f Le cos), weight
// balance(p_light, M, p_bsdf, N) p^ / p_light, one weighted-reservoir draw per candidate
// (RIS_Reservoir.h add_one_candidate: M++, w_sum += w, keep if u < w / w_sum). 'eval(wi, pdf)'
// evaluates the BSDF (f without the cosine) and its pdf.
struct RisPick
{
    V3 point, contrib, dir;  // contrib = f Le cos of the kept candidate
    float target, dist, wsum;
    bool kept;
};

template <class Eval>
__device__ __forceinline__ RisPick ris_light_candidates(const SceneView& s, const RenderConst& rc, Pcg32& rng, V3 P, V3 ns,
                                                        int M, int N, Eval eval)
{
    RisPick r;
    r.kept = false;
    r.wsum = 0.0f;
    r.target = 0.0f;
    r.dist = 0.0f;
    r.point = r.contrib = r.dir = v3(0.0f);
    for (int i = 0; i < M; i++)
    {
        const LightSample ls = sample_light(s, rc, rng);
        float w = 0.0f, target = 0.0f, dist = 0.0f;
        V3 c = v3(0.0f), wi = v3(0.0f);
        if (ls.pdf_area > 0.0f)
        {
            const V3 tl = ls.point - P;
            dist = length(tl);
            wi = tl / dist;
            const float cos_l = fmaxf(0.0f, dot(ls.normal, -wi));
            const float cos_p = fabsf(dot(ns, wi));
            if (cos_p > 0.0f && cos_l > 1.0e-6f)
            {
                float p_bsdf;
                const V3 f = eval(wi, p_bsdf);
                c = f * ls.emission * cos_p;
                target = luminance(c);
                const float p_light = area_to_solid_angle_pdf(ls.pdf_area, dist, cos_l);
                w = balance_counts(p_light, (float)M, p_bsdf, (float)N) * target / p_light;
            }
        }
        r.wsum += w;
        if (rng.next() < w / r.wsum)
        {
            r.kept = true;
            r.point = ls.point;
            r.contrib = c;
            r.dir = wi;
            r.dist = dist;
            r.target = target;
        }
    }
    return r;
}

// A BSDF sample draws its random numbers from a Xorshift32 generator (the reference's generator,
// src/HostDeviceCommon/Xorshift.h): with PCG paths one seeded by the path's stream, so the same
// numbers can be replayed through the reference's own BSDF; under GBPT_RNG_REFERENCE the path's own
// generator, as the reference's BSDF samplers take it, continued by bsdf_rng_done afterwards.
__device__ __forceinline__ bsdf::Xorshift32 bsdf_rng(Pcg32& rng)
{
    if (rng.inc == 0) return bsdf::Xorshift32{(uint32_t)rng.state};
    uint32_t seed = rng.next_u32();
    return bsdf::Xorshift32{seed != 0u ? seed : 0x9E3779B9u};
}
__device__ __forceinline__ void bsdf_rng_done(Pcg32& rng, const bsdf::Xorshift32& xr)
{
    if (rng.inc == 0) rng.state = xr.state;
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
