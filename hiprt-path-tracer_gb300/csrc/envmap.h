// Environment-map lighting on the device: RGB9E5 texels, equirectangular lookups, importance
// sampling by alias table or CDF search, the pdf of a direction, and the radiance a miss sees.
//
// Restates src/Device/includes/LightSampling/Envmap.h:27-249 (eval_envmap_no_pdf,
// envmap_cdf_search, envmap_sample, envmap_eval, sample_environment_map_with_mis),
// src/Device/includes/Texture.h:209-240 (sample_environment_map_texture) and
// src/Device/includes/PathTracing.h:122-169 (path_tracing_miss_gather_envmap). The reference's
// estimator is kept as it is, including two of its properties:
//   - a sampled texel yields the direction of its (u, v) = (x/W, y/H) corner, and the radiance and
//     pdf of that sample are read at texel (floor(u (W-1)), floor(v (H-1))) — the neighbour below
//     and left of it for x, y >= 1;
//   - envmap_eval takes theta of the pdf from the world direction, before the envmap rotation.
// Two guards that change nothing for valid inputs: the sine of asin is clamped to [-1, 1] and the
// texel indices to the image, so a direction that normalisation left a hair outside the unit
// sphere cannot index outside the texels; the alias index is split into (x, y) by integer division
// (the reference's float division agrees below 2^24 texels).
#pragma once

#include "render_common.h"

namespace gbpt {

constexpr float kEnvInv2Pi = 0.15915494309189533577f;
constexpr float kEnvInvPi = 0.31830988618379067154f;
constexpr float kEnvTwoPiSquared = 19.73920880217871723767f;

#ifdef __CUDACC__

// RGB9E5 (R9G9B9E5_SHAREDEXP, RGBE9995Packed::unpack): three 9-bit mantissas scaled by 2^(E - 24)
__device__ __forceinline__ V3 rgb9e5_unpack(uint32_t t)
{
    const float scale = __uint_as_float((uint32_t)((int)(t >> 27) - 24 + 127) << 23);
    return v3((float)(t & 0x1FFu) * scale, (float)((t >> 9) & 0x1FFu) * scale, (float)((t >> 18) & 0x1FFu) * scale);
}

__device__ __forceinline__ V3 mat3_x(const float* m, V3 d)
{
    return v3(m[0] * d.x + m[1] * d.y + m[2] * d.z, m[3] * d.x + m[4] * d.y + m[5] * d.z,
              m[6] * d.x + m[7] * d.y + m[8] * d.z);
}

__device__ __forceinline__ V3 env_texel(const EnvView& e, int x, int y)
{
    x = min(max(x, 0), e.width - 1);
    y = min(max(y, 0), e.height - 1);
    return rgb9e5_unpack(__ldg(e.texels + (int64_t)y * e.width + x)) * e.intensity;
}

// sample_environment_map_texture: nearest texel of (u (W-1), v (H-1)), or bilinear between the
// four texels around it; scaled by the intensity
__device__ __forceinline__ V3 env_texture(const EnvView& e, float u, float v)
{
    const float fx = u * (float)(e.width - 1), fy = v * (float)(e.height - 1);
    if (!e.bilinear) return env_texel(e, (int)fx, (int)fy);
    const int x0 = (int)fx, y0 = (int)fy;
    const float tx = fx - floorf(fx), ty = fy - floorf(fy);
    const int x1 = min(x0 + 1, e.width - 1), y1 = min(y0 + 1, e.height - 1);
    const V3 c00 = env_texel(e, x0, y0), c10 = env_texel(e, x1, y0);
    const V3 c01 = env_texel(e, x0, y1), c11 = env_texel(e, x1, y1);
    const V3 a = c00 * (1.0f - tx) + c10 * tx;
    const V3 b = c01 * (1.0f - tx) + c11 * tx;
    return a * (1.0f - ty) + b * ty;
}

// eval_envmap_no_pdf: radiance arriving from world direction d
__device__ __forceinline__ V3 env_lookup(const EnvView& e, V3 d)
{
    const V3 r = mat3_x(e.to_env, d);
    const float u = 0.5f + atan2f(r.z, r.x) * kEnvInv2Pi;
    const float v = 0.5f + asinf(fminf(1.0f, fmaxf(-1.0f, r.y))) * kEnvInvPi;
    return env_texture(e, u, v);
}

// luminance-proportional texel pdf converted to solid angle (Envmap.h:120-131)
__device__ __forceinline__ float env_pdf(const EnvView& e, V3 L, float sin_theta)
{
    float pdf = luminance(L) / (e.total_sum * e.intensity);
    pdf *= (float)(e.width * e.height);
    return pdf / (kEnvTwoPiSquared * sin_theta);
}

struct EnvSample
{
    V3 dir, L;
    float pdf;
};

// envmap_cdf_search: the first row whose running sum at its last texel exceeds 'value', then the
// first texel of that row whose running sum exceeds it
__device__ __forceinline__ void env_cdf_search(const EnvView& e, float value, int& x, int& y)
{
    int lo = 0, hi = e.height - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (value < __ldg(e.cdf + (int64_t)mid * e.width + (e.width - 1)))
            hi = mid;
        else
            lo = mid + 1;
    }
    y = min(lo, e.height - 1);
    lo = 0;
    hi = e.width - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (value < __ldg(e.cdf + (int64_t)y * e.width + mid))
            hi = mid;
        else
            lo = mid + 1;
    }
    x = min(lo, e.width - 1);
}

// envmap_sample: texel by the alias table (index draw, then the alias test) or by the CDF (one
// draw), direction of its corner, radiance and pdf
__device__ __forceinline__ EnvSample env_sample(const EnvView& e, Pcg32& rng)
{
    int x, y;
    if (e.sampling == GBPT_ENVMAP_BINARY_SEARCH)
        env_cdf_search(e, rng.next() * e.total_sum, x, y);
    else
    {
        const int n = e.width * e.height;
        int i = rng.index(n);
        const uint2 pa = __ldg(e.alias + i);
        if (rng.next() > __uint_as_float(pa.x)) i = (int)pa.y;
        y = i / e.width;
        x = i - y * e.width;
    }
    const float u = (float)x / (float)e.width, v = (float)y / (float)e.height;
    const float phi = u * kTwoPi;
    const float theta = fmaxf(1.0e-5f, v * kPi);
    const float ct = cosf(theta), st = sinf(theta);
    EnvSample s;
    s.dir = mat3_x(e.to_world, v3(-st * cosf(phi), -ct, -st * sinf(phi)));
    s.L = env_texture(e, u, v);
    s.pdf = env_pdf(e, s.L, st);
    return s;
}

// envmap_eval: radiance from world direction d and the pdf of sampling it
__device__ __forceinline__ V3 env_eval(const EnvView& e, V3 d, float& pdf)
{
    const V3 L = env_lookup(e, d);
    const float theta = acosf(-d.y);
    pdf = env_pdf(e, L, sinf(theta));
    return L;
}

// importance-sampled envmap direct lighting is on at shaded vertices
__device__ __forceinline__ bool env_sampled(const EnvView& e)
{
    return e.ambient == GBPT_AMBIENT_ENVMAP && e.sampling != GBPT_ENVMAP_NO_SAMPLING && e.intensity > 0.0f;
}

// path_tracing_miss_gather_envmap: radiance a ray of the given bounce sees when it leaves the scene
// (times the path throughput tp). With envmap sampling only camera rays see the envmap (the
// vertices' direct lighting covers the rest); camera rays see the unscaled texels unless
// scale_background is set.
__device__ __forceinline__ V3 env_miss(const EnvView& e, V3 d, int bounce, V3 tp)
{
    if (e.ambient == GBPT_AMBIENT_UNIFORM) return v3(e.uniform[0], e.uniform[1], e.uniform[2]) * tp;
    if (e.ambient != GBPT_AMBIENT_ENVMAP || !(e.intensity > 0.0f)) return v3(0.0f);
    const bool sampled = e.sampling != GBPT_ENVMAP_NO_SAMPLING;
    if (sampled && bounce > 0) return v3(0.0f);
    V3 c = env_lookup(e, d);
    if (!e.scale_background && (sampled || bounce == 0)) c = c / e.intensity;
    return c * tp;
}

// Envmap direct lighting at a vertex (sample_environment_map_with_mis, Envmap.h:173-249): an
// envmap sample weighted against the BSDF pdf (light_ok: the material can be light-sampled) and a
// separate BSDF sample weighted against the envmap pdf, each visible through an any-hit ray to
// 1e35. eval(wi, pdf) -> f; sample(wi, pdf) -> f draws a BSDF direction.
struct EnvDirect
{
    bool want_l = false, want_b = false;
    V3 dir_l, dir_b;
    V3 c_l, c_b;
};

template <class Eval, class Sample>
__device__ __forceinline__ EnvDirect env_direct(const EnvView& e, Pcg32& rng, V3 ns, V3 tp, bool light_ok, Eval eval,
                                                Sample sample)
{
    EnvDirect r;
    const EnvSample es = env_sample(e, rng);
    if (light_ok)
    {
        const float cosine = dot(ns, es.dir);
        if (es.pdf > 0.0f && cosine > 0.0f)
        {
            float bsdf_pdf;
            const V3 f = eval(es.dir, bsdf_pdf);
            const float mis = e.bsdf_mis ? balance_heuristic(es.pdf, bsdf_pdf) : 1.0f;
            const V3 c = tp * (f * cosine * mis * es.L / es.pdf);
            if (!is_black(c))
            {
                r.want_l = true;
                r.dir_l = es.dir;
                r.c_l = c;
            }
        }
    }
    if (e.bsdf_mis)
    {
        V3 wi;
        float pdf;
        const V3 f = sample(wi, pdf);
        if (pdf > 0.0f)
        {
            const float cosine = fabsf(dot(ns, wi));
            float env_p;
            const V3 L = env_eval(e, wi, env_p);
            if (env_p > 0.0f)
            {
                const V3 c = tp * (L * balance_heuristic(pdf, env_p) * cosine * f / pdf);
                if (!is_black(c))
                {
                    r.want_b = true;
                    r.dir_b = wi;
                    r.c_b = c;
                }
            }
        }
    }
    return r;
}

#endif  // __CUDACC__

}  // namespace gbpt
