/*
 * TEST INFRASTRUCTURE ONLY — C entry points into the reference's OWN environment-map code,
 * compiled from the reference's sources where they lie (oracle/Makefile, target 'ref'), behind the
 * clean-room shim headers in oracle/shim/. Output goes to oracle/_ref/ (git-ignored). Used by
 * tests/golden/make_envmap_golden.py to write the golden vectors that pin this project's envmap
 * oracle (oracle/pt_oracle.cpp) and, through it, the GPU kernels.
 *
 * Calls, unmodified: RGBE9995Packed::pack / unpack (src/HostDeviceCommon/Packing.h:441-485),
 * eval_envmap_no_pdf, envmap_cdf_search, envmap_sample and envmap_eval
 * (src/Device/includes/LightSampling/Envmap.h:27-170), which read texels through
 * sample_environment_map_texture (src/Device/includes/Texture.h:209-240).
 * Compile-time options: EnvmapSamplingStrategy at its default (ESS_ALIAS_TABLE);
 * EnvmapSamplingDoBilinearFiltering = REF_ENV_BILINEAR (the Makefile builds libref_env.so with 0,
 * the reference's default, and libref_env_bilinear.so with 1). Only the C entry points are
 * exported, so the two libraries' inline reference functions stay apart.
 *
 * Envmap parameters: texels (RGB9E5 words), CDF, alias probabilities and indices, width, height,
 * intensity, total luminance sum, and the envmap-to-world / world-to-envmap rotations as row-major
 * 3x3 matrices (d' = M d).
 */
#include "HostDeviceCommon/KernelOptions/KernelOptions.h"

#ifndef REF_ENV_BILINEAR
#define REF_ENV_BILINEAR 0
#endif
#undef EnvmapSamplingDoBilinearFiltering
#if REF_ENV_BILINEAR
#define EnvmapSamplingDoBilinearFiltering KERNEL_OPTION_TRUE
#else
#define EnvmapSamplingDoBilinearFiltering KERNEL_OPTION_FALSE
#endif

#include "Device/includes/LightSampling/Envmap.h"

#include <cstdint>
#include <cstring>

#define REF_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

struct RefEnv
{
    const uint32_t* texels;
    const float* cdf;
    const float* probas;
    const int32_t* alias;
    int32_t width, height;
    float intensity, total_sum;
    float to_world[9], to_env[9];
};

WorldSettings world(const RefEnv* e)
{
    WorldSettings ws;
    ws.ambient_light_type = AmbientLightType::ENVMAP;
    ws.envmap_width = (unsigned int)e->width;
    ws.envmap_height = (unsigned int)e->height;
    ws.envmap_intensity = e->intensity;
    ws.envmap = reinterpret_cast<RGBE9995Packed*>(const_cast<uint32_t*>(e->texels));
    ws.envmap_total_sum = e->total_sum;
    ws.envmap_cdf = const_cast<float*>(e->cdf);
    ws.envmap_alias_table.alias_table_probas = const_cast<float*>(e->probas);
    ws.envmap_alias_table.alias_table_alias = const_cast<int*>(e->alias);
    ws.envmap_alias_table.size = (unsigned int)(e->width * e->height);
    ws.envmap_alias_table.sum_elements = e->total_sum;
    // float3x3 holds columns (m[c][r]); matrix_X_vec computes sum_c m[c][r] v_c
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
        {
            ws.envmap_to_world_matrix.m[c][r] = e->to_world[3 * r + c];
            ws.world_to_envmap_matrix.m[c][r] = e->to_env[3 * r + c];
        }
    return ws;
}

}  // namespace

REF_EXPORT void ref_env_rgbe_pack(const float* rgb, int n, uint32_t* out)
{
    for (int i = 0; i < n; i++)
    {
        RGBE9995Packed p;
        p.pack(ColorRGB32F(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]));
        std::memcpy(out + i, &p, sizeof(uint32_t));
    }
}

REF_EXPORT void ref_env_rgbe_unpack(const uint32_t* in, int n, float* rgb)
{
    for (int i = 0; i < n; i++)
    {
        RGBE9995Packed p;
        std::memcpy(&p, in + i, sizeof(uint32_t));
        const ColorRGB32F c = p.unpack();
        rgb[3 * i] = c.r;
        rgb[3 * i + 1] = c.g;
        rgb[3 * i + 2] = c.b;
    }
}

// eval_envmap_no_pdf for n world directions
REF_EXPORT void ref_env_lookup(const RefEnv* e, const float* dirs, int n, float* rgb)
{
    const WorldSettings ws = world(e);
    for (int i = 0; i < n; i++)
    {
        const ColorRGB32F c = eval_envmap_no_pdf(ws, make_float3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
        rgb[3 * i] = c.r;
        rgb[3 * i + 1] = c.g;
        rgb[3 * i + 2] = c.b;
    }
}

// envmap_eval: radiance and solid-angle pdf of n world directions
REF_EXPORT void ref_env_eval(const RefEnv* e, const float* dirs, int n, float* rgb, float* pdf)
{
    HIPRTRenderData rd;
    rd.world_settings = world(e);
    for (int i = 0; i < n; i++)
    {
        float p = 0.0f;
        const ColorRGB32F c = envmap_eval(rd, make_float3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]), p);
        rgb[3 * i] = c.r;
        rgb[3 * i + 1] = c.g;
        rgb[3 * i + 2] = c.b;
        pdf[i] = p;
    }
}

// envmap_sample (alias-table strategy) from a Xorshift32 generator seeded with seeds[i]; also
// returns the generator's two draws: the table index and the alias-test number
REF_EXPORT void ref_env_sample(const RefEnv* e, const uint32_t* seeds, int n, float* dir, float* rgb, float* pdf,
                               int32_t* index, float* u)
{
    const WorldSettings ws = world(e);
    for (int i = 0; i < n; i++)
    {
        Xorshift32Generator g(seeds[i]);
        Xorshift32Generator g2 = g;
        float3 d;
        float p = 0.0f;
        const ColorRGB32F c = envmap_sample(ws, d, p, g);
        dir[3 * i] = d.x;
        dir[3 * i + 1] = d.y;
        dir[3 * i + 2] = d.z;
        rgb[3 * i] = c.r;
        rgb[3 * i + 1] = c.g;
        rgb[3 * i + 2] = c.b;
        pdf[i] = p;
        index[i] = g2.random_index((int)(e->width * e->height));
        u[i] = g2();
    }
}

// envmap_cdf_search for n values in [0, total_sum)
REF_EXPORT void ref_env_cdf_search(const RefEnv* e, const float* values, int n, int32_t* xy)
{
    const WorldSettings ws = world(e);
    for (int i = 0; i < n; i++)
    {
        int x = 0, y = 0;
        envmap_cdf_search(ws, values[i], x, y);
        xy[2 * i] = x;
        xy[2 * i + 1] = y;
    }
}
